// Cell grid build (counting sort) and the gather / scatter between the caller's
// particle order and the cell-sorted working order, per scene.
//
// Reference: Ngrid.clear_node / encode / mem_shift / fill_node, sph_obj.py:295-323,
// and the per-step bookkeeping of sph.py:22-47, 265-286.  Differences by design:
// the cell offsets are an ordered exclusive scan instead of an atomic bump
// (mem_shift), and particles inside a cell are ordered by particle id, so the
// layout -- and every FP32 sum over it -- is deterministic.
#include <cuda_runtime.h>

#include "ctx.h"

namespace tsph {

// ----------------------------------------------------------------------------- CFL
// cfl_condition, sph.py:41-47, per scene: dt = part_size / cs, lowered to
// part_size / |v| * cfl_factor for |v| > 1e-4.  part_size / v * cfl is monotone
// in v, so the minimum over particles is attained at max |v|.
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_cfl(KConst k, const float *__restrict__ vel, int64_t n) {
    pdl_entry();
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * kBlock;
    // each warp keeps its running maximum for the scene it last saw and issues
    // one atomic when the scene changes (and at the end): one atomic per warp
    // for a one-scene context instead of one per warp and iteration
    int wsc = -1;
    float wmax = 0.f;
    for (int64_t base = blockIdx.x * (int64_t)kBlock; base < n; base += stride) {
        const int64_t i = base + threadIdx.x;
        const bool act = i < n;
        float vn = 0.f;
        int sc = -1;
        if (act) {
            float s = 0.f;
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                const float v = vel[i * DIM + d];
                s += v * v;
            }
            vn = sqrtf(s);
            if (!(vn > 1e-4f)) vn = 0.f;  // NaN norms fail the test, as in the reference
            sc = k.f_user_scene[i];
        }
        const int sc0 = __shfl_sync(0xffffffffu, sc, 0);
        if (sc0 < 0) continue;  // no particle left in this warp
        if (__all_sync(0xffffffffu, !act || sc == sc0)) {
            float m = vn;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
            if (sc0 != wsc) {
                if (lane == 0 && wsc >= 0 && wmax > 0.f) atomicMax(&k.ss[wsc].vmax_bits, __float_as_uint(wmax));
                wsc = sc0;
                wmax = m;
            } else {
                wmax = fmaxf(wmax, m);
            }
        } else if (act && vn > 0.f) {
            atomicMax(&k.ss[sc].vmax_bits, __float_as_uint(vn));
        }
    }
    if (lane == 0 && wsc >= 0 && wmax > 0.f) atomicMax(&k.ss[wsc].vmax_bits, __float_as_uint(wmax));
    if (last_block_done(&k.dg->ticket[kGtCfl], gridDim.x)) {
        for (int s = threadIdx.x; s < k.n_scenes; s += kBlock) {
            const SceneConst &c = k.sc[s];
            float dt = __fdiv_rn(c.part_size, (float)c.cs);
            const float vm = __uint_as_float(atomicExch(&k.ss[s].vmax_bits, 0u));
            if (vm > 1e-4f) dt = fminf(dt, __fmul_rn(__fdiv_rn(c.part_size, vm), c.cfl));
            k.sp[s].dt = dt;
            k.sp[s].time_count += (double)dt;
        }
        if (threadIdx.x == 0) k.dg->ticket[kGtCfl] = 0;
    }
}

// ----------------------------------------------------------------------------- encode
// Ngrid.encode, sph_obj.py:300-306: structured cell, scene-local linear code,
// count in the scene's range of the global grid.  A particle without a valid
// code gets a rank in its scene's tail.
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_encode(KConst k, tsph_set U, int bound, int *__restrict__ count,
                                                   int *__restrict__ slot) {
    pdl_entry();
    const int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (i >= U.n) return;
    const int sc = bound ? k.b_user_scene[i] : k.f_user_scene[i];
    Geo g;
    g.load(k.sc[sc], k.R);
    float4 p = make_float4(U.pos[i * DIM], U.pos[i * DIM + 1], DIM == 3 ? U.pos[i * DIM + 2] : 0.f, 0.f);
    bool ok;
    long long code = cell_code<DIM>(p, g, ok);
    const float c[3] = {p.x, p.y, p.z};
#pragma unroll
    for (int d = 0; d < DIM; ++d)
        U.neighb_cell_structured_seq[i * DIM + d] = ok ? (int)floorf(__fdiv_rn(c[d] - g.lb[d], g.h)) : 0;
    U.neighb_cell_seq[i] = (int)code;
    int s;
    if (ok && code > 0 && code < g.node_num) {
        s = atomicAdd(count + g.cbase + code, 1);
    } else {
        s = -1 - atomicAdd(bound ? &k.ss[sc].b_tail : &k.ss[sc].f_tail, 1);
        atomicOr(&k.ss[sc].status, ok ? TSPH_ST_OUTSIDE_GRID : (TSPH_ST_NONFINITE_POS | TSPH_ST_OUTSIDE_GRID));
    }
    slot[i] = s;
}

// ----------------------------------------------------------------------------- scan
// Exclusive scan of the cell counts in two launches (blockIdx.y selects the
// fluid (0) or boundary (1) grid; 4096 cells per block):
//   k_scan_reduce: each block's total; the grid's last block to finish scans
//     the totals in place (a ticket, no block waits for another);
//   k_scan_down: each block scans its cells again and adds its offset; the last
//     block over both grids derives the per-scene shifts from the finished
//     starts.
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

struct ScanArgs {
    const int *count[2];
    int *start[2];
    int *blocks[2];
    int64_t n;
};

__device__ __forceinline__ int block_excl_scan(int v, int *sh, int &total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        int t = (lane < kScanThreads / 32) ? sh[lane] : 0;
        int u = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, u, o);
            if (lane >= o) u += y;
        }
        sh[lane] = u - t;           // exclusive prefix of warp totals
        if (lane == 31) sh[32] = u;  // block total
    }
    __syncthreads();
    total = sh[32];
    int r = sh[w] + x - v;
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(ScanArgs a, int nblocks, unsigned int *tickets) {
    pdl_entry();
    __shared__ int sh[33];
    const int g = blockIdx.y;
    const int64_t base = blockIdx.x * (int64_t)kScanTile + threadIdx.x * kScanItems;
    int sum = 0;
#pragma unroll
    for (int t = 0; t < kScanItems; ++t)
        if (base + t < a.n) sum += a.count[g][base + t];
    int total;
    block_excl_scan(sum, sh, total);
    if (threadIdx.x == 0) a.blocks[g][blockIdx.x] = total;
    if (!last_block_done(&tickets[g], (unsigned int)nblocks)) return;
    // this grid's block totals -> exclusive offsets, in place; [nblocks] = total
    int carry = 0;
    for (int b0 = 0; b0 < nblocks; b0 += kScanTile) {
        int v[kScanItems];
        int s = 0;
        const int i0 = b0 + threadIdx.x * kScanItems;
#pragma unroll
        for (int t = 0; t < kScanItems; ++t) {
            v[t] = (i0 + t < nblocks) ? __ldcg(&a.blocks[g][i0 + t]) : 0;
            s += v[t];
        }
        int tot;
        int run = block_excl_scan(s, sh, tot) + carry;
#pragma unroll
        for (int t = 0; t < kScanItems; ++t) {
            if (i0 + t < nblocks) a.blocks[g][i0 + t] = run;
            run += v[t];
        }
        carry += tot;
    }
    if (threadIdx.x == 0) {
        a.blocks[g][nblocks] = carry;
        tickets[g] = 0;
    }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_down(ScanArgs a, int nblocks, KConst k, unsigned int *ticket) {
    pdl_entry();
    __shared__ int sh[33];
    const int g = blockIdx.y;
    const int64_t base = blockIdx.x * (int64_t)kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems];
    int sum = 0;
#pragma unroll
    for (int t = 0; t < kScanItems; ++t) {
        v[t] = (base + t < a.n) ? a.count[g][base + t] : 0;
        sum += v[t];
    }
    int total;
    int run = block_excl_scan(sum, sh, total) + a.blocks[g][blockIdx.x];
#pragma unroll
    for (int t = 0; t < kScanItems; ++t) {
        if (base + t < a.n) a.start[g][base + t] = run;
        run += v[t];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) a.start[g][a.n] = a.blocks[g][nblocks];
    if (!last_block_done(ticket, 2u * (unsigned int)nblocks)) return;
    // per scene: in-grid counts and the shift from global scan positions to the
    // scene's sorted slots
    for (int s = threadIdx.x; s < k.n_scenes; s += blockDim.x) {
        const SceneConst &c = k.sc[s];
        SceneStep &st = k.ss[s];
        const int f0 = __ldcg(&a.start[0][c.cbase]), f1 = __ldcg(&a.start[0][c.cbase + c.node_num]);
        const int b0 = __ldcg(&a.start[1][c.cbase]), b1 = __ldcg(&a.start[1][c.cbase + c.node_num]);
        st.f_in = f1 - f0;
        st.b_in = b1 - b0;
        st.f_shift = c.f_slot - f0;
        st.b_shift = c.b_slot - b0;
    }
    if (threadIdx.x == 0) *ticket = 0;
}

// ----------------------------------------------------------------------------- scatter
__global__ void __launch_bounds__(kBlock) k_scatter(KConst k, int bound, int64_t n, const int *__restrict__ code,
                                                    const int *__restrict__ slot, const int *__restrict__ start,
                                                    int *__restrict__ perm) {
    pdl_entry();
    const int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (i >= n) return;
    const int sc = bound ? k.b_user_scene[i] : k.f_user_scene[i];
    const SceneConst &c = k.sc[sc];
    const SceneStep &st = k.ss[sc];
    const int sl = slot[i];
    long long s;
    if (sl >= 0) s = (long long)start[c.cbase + code[i]] + (bound ? st.b_shift : st.f_shift) + sl;
    else s = (bound ? c.b_slot + st.b_in : c.f_slot + st.f_in) + (-1 - sl);
    perm[s] = (int)i;
}

// Sorted slot of the particle `pid` found at unsorted slot range [beg, end) of
// its cell (or of its scene's tail of particles without a valid cell): a cell's
// particles are ordered by id, so its slot is the range's first slot plus the
// number of the range's particles with a smaller id.
__device__ __forceinline__ int64_t sorted_slot(const int *__restrict__ perm_u, int64_t beg, int64_t end, int pid) {
    int r = 0;
    for (int64_t a = beg; a < end; ++a) r += perm_u[a] < pid;
    return beg + r;
}

// The slot range of the cell (in-grid particles, slots [slot0, slot0 + n_in))
// or of the scene's tail that holds the particle at unsorted slot u; `shift`
// maps the grid's scan positions to the scene's slots, as in k_scatter.
__device__ __forceinline__ void slot_range(const SceneConst &c, long long shift, const int *__restrict__ start,
                                           int64_t u, int64_t slot0, int32_t n_in, int32_t n_tail, int code,
                                           int64_t &beg, int64_t &end) {
    if (u - slot0 < n_in) {
        beg = start[c.cbase + code] + shift;
        end = start[c.cbase + code + 1] + shift;
    } else {
        beg = slot0 + n_in;
        end = beg + n_tail;
    }
}

// ----------------------------------------------------------------------------- gather
// Copies the caller-order state into the sorted working arrays; v_adv = vel
// (SPH_vel_2_vel_adv, sph.py:253-256).  X / psi0 follow the solver aliases,
// sph_obj.py:65-73.
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_gather_fluid(KConst k, tsph_set U, FluidBuf F) {
    pdl_entry();
    const int64_t u = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (u >= F.cap) return;
    const int sc = k.f_chunk_scene[u / kChunk];
    const SceneConst &c = k.sc[sc];
    if (u - c.f_slot >= c.f_n) return;
    const SceneStep &st = k.ss[sc];
    const int pid = F.perm_u[u];
    int64_t beg, end;
    slot_range(c, st.f_shift, F.start, u, c.f_slot, st.f_in, st.f_tail, U.neighb_cell_seq[pid], beg, end);
    const int64_t s = sorted_slot(F.perm_u, beg, end, pid);
    F.perm[s] = pid;
    F.inv[pid] = (int)s;
    const float *p = U.pos + (int64_t)pid * DIM;
    const float *v = U.vel + (int64_t)pid * DIM;
    const float m = U.mass[pid], V = U.rest_volume[pid], r0 = U.rest_density[pid];
    F.pos[s] = make_float4(p[0], p[1], DIM == 3 ? p[2] : 0.f, k.vfsph ? V : m);
    F.mv[s] = make_float2(m, V);
    F.rho0[s] = r0;
    F.mpsi[s] = make_float4(m, 0.f, k.vfsph ? 1.f : r0, 0.f);
    F.vadv[s] = make_float4(v[0], v[1], DIM == 3 ? v[2] : 0.f, 0.f);
    for (int q = 0; q < k.P; ++q) F.vf[q * F.cap + s] = U.volume_frac[(int64_t)pid * k.P + q];
}

template <int DIM>
__global__ void __launch_bounds__(kBlock) k_gather_bound(KConst k, tsph_set U, BoundBuf B) {
    pdl_entry();
    const int64_t u = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (u >= B.cap) return;
    const int sc = k.b_chunk_scene[u / kChunk];
    const SceneConst &c = k.sc[sc];
    if (u - c.b_slot >= c.b_n) return;
    const SceneStep &st = k.ss[sc];
    const int pid = B.perm_u[u];
    int64_t beg, end;
    slot_range(c, st.b_shift, B.start, u, c.b_slot, st.b_in, st.b_tail, U.neighb_cell_seq[pid], beg, end);
    const int64_t s = sorted_slot(B.perm_u, beg, end, pid);
    B.perm[s] = pid;
    B.inv[pid] = (int)s;
    const float *p = U.pos + (int64_t)pid * DIM;
    const float *va = U.vel_adv + (int64_t)pid * DIM;
    const float m = U.mass[pid], V = U.rest_volume[pid];
    const float4 np = make_float4(p[0], p[1], DIM == 3 ? p[2] : 0.f, k.vfsph ? V : m);
    const float4 op = B.pos[s];
    const float2 omv = B.mv[s];
    // the slot's previous contents: equal everywhere means the same sorted
    // order, grid and boundary-boundary sums as the previous gather.  A change
    // also drops the kept sums for good, so that a later step cannot take them
    // after a call that gathered without a density sweep (the neighbour stats)
    const bool same = __float_as_uint(op.x) == __float_as_uint(np.x) && __float_as_uint(op.y) == __float_as_uint(np.y) &&
                      __float_as_uint(op.z) == __float_as_uint(np.z) && __float_as_uint(op.w) == __float_as_uint(np.w) &&
                      __float_as_uint(omv.x) == __float_as_uint(m) && __float_as_uint(omv.y) == __float_as_uint(V);
    // one store per warp that saw a change (a warp lies in one scene's chunk),
    // none once the flag is up: every slot differs in a first gather or under
    // a moving boundary, and the stores would all go to one word
    const unsigned int changed = __ballot_sync(__activemask(), !same);
    if (changed && (threadIdx.x & 31) == __ffs(changed) - 1 && !__ldcg(&k.ss[sc].b_dirty)) {
        k.ss[sc].b_dirty = 1;
        k.sp[sc].bb_valid = 0;
    }
    B.pos[s] = np;
    B.mv[s] = make_float2(m, V);
    B.vadv[s] = make_float4(va[0], va[1], DIM == 3 ? va[2] : 0.f, 0.f);
    B.kappa[s] = U.psi_adv[pid];  // divided by alpha once alpha is known
}

// ----------------------------------------------------------------------------- update
// SPH_update_volume_frac, SPH_update_mass, SPH_update_pos and SPH_update_energy
// (sph.py:265-286, 375-379) in the caller's particle order: each thread gathers
// its particle's sorted state (inv) so that the ~20 per-particle result arrays
// are written coalesced.  Blocks walk each scene's caller range padded to whole
// blocks.  Energies: per-particle FP32 terms, FP64 block sums, the scene's
// blocks summed in order by the scene's last block.
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_update_fluid(KConst k, tsph_set U, FluidBuf F,
                                                         const int *__restrict__ bstart, double *partials, int fbm,
                                                         int st_on) {
    pdl_entry();
    __shared__ double sh[kBlock / 32];
    const int sc = k.f_ublock_scene[blockIdx.x];
    const SceneConst &c = k.sc[sc];
    SceneStep &st = k.ss[sc];
    const int64_t local = (blockIdx.x - c.f_ublk0) * (int64_t)kBlock + threadIdx.x;
    double ke = 0.0, pe = 0.0;
    if (local < c.f_n) {
        const int64_t pid = c.f_user + local;
        const int64_t s = F.inv[pid];
        const float dt = k.sp[sc].dt;
        const float4 v = F.vadv[st.cur * F.cap + s];
        const float4 p = F.pos[s];
        const float4 dn = F.dens[s];
        const float V = F.mv[s].y;
        const int flagged = fbm ? (F.flagpass[s] != 0) : 0;
        float rho0 = 0.f;
        for (int q = 0; q < k.P; ++q) {
            float vf = F.vf[q * F.cap + s];
            if (fbm) {
                const float t = F.vftmp[q * F.cap + s];
                if (!flagged) vf += t;
                U.volume_frac[pid * k.P + q] = vf;
                U.volume_frac_tmp[pid * k.P + q] = t;
            }
            rho0 += c.rho_phase[q] * vf;
        }
        const float m = rho0 * V;
        const float np[3] = {p.x + v.x * dt, p.y + v.y * dt, p.z + v.z * dt};
        const float vv[3] = {v.x, v.y, v.z};
        const float4 acc = F.acc[s];
        const float aa[3] = {acc.x, acc.y, acc.z};
        const float4 a1 = F.a1[s];
        const float a1v[3] = {a1.x, a1.y, a1.z};
        const int64_t b = pid * DIM;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            U.pos[b + d] = np[d];
            U.vel[b + d] = vv[d];
            U.vel_adv[b + d] = vv[d];
            U.acce_adv[b + d] = aa[d];
            U.alpha_1[b + d] = a1v[d];
        }
        if (st_on) {
            const float4 nr = F.normal[s];
            const float nrv[3] = {nr.x, nr.y, nr.z};
#pragma unroll
            for (int d = 0; d < DIM; ++d) U.normal[b + d] = nrv[d];
        }
        if (fbm) {
            const float4 fa = F.facc[s];
            const float fav[3] = {fa.x, fa.y, fa.z};
#pragma unroll
            for (int d = 0; d < DIM; ++d) U.acce[b + d] = fav[d];
            for (int q = 0; q < k.P; ++q) {
                const float4 dv = F.drift[s * k.P + q];
                const float dvv[3] = {dv.x, dv.y, dv.z};
#pragma unroll
                for (int d = 0; d < DIM; ++d) U.drift_vel[(pid * k.P + q) * DIM + d] = dvv[d];
            }
            U.fbm_zeta[pid] = F.zeta[s];
        }
        U.flag[pid] = flagged;
        U.mass[pid] = m;
        U.rest_density[pid] = rho0;
        U.W[pid] = dn.x;
        U.sph_density[pid] = dn.y;
        U.sph_compression[pid] = dn.z;
        U.psi_adv[pid] = F.psiadv[s];
        if (F.wcp && U.pressure) U.pressure[pid] = F.wcp[s].x;
        U.alpha[pid] = a1.w;  // alpha, stored beside alpha_1 by the density sweep
        U.alpha_2[pid] = dn.w;
        if (s - c.f_slot < st.f_in) {
            // slot in the reference's combined grid: cell offset over both sets, fluid first
            const int code = U.neighb_cell_seq[pid];
            U.neighb_in_cell_seq[pid] = (int)(s - st.f_shift) + bstart[c.cbase + code];
        }
        float v2 = 0.f;
#pragma unroll
        for (int d = 0; d < DIM; ++d) v2 += vv[d] * vv[d];
        ke = (double)(0.5f * m * v2);
        pe = (double)(-m * c.g[1] * (np[1] - c.lb[1]));
    }
    const double bke = block_sum<kBlock>(ke, sh);
    const double bpe = block_sum<kBlock>(pe, sh);
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = bke;
        partials[2 * blockIdx.x + 1] = bpe;
    }
    const unsigned int nblk = (unsigned int)c.f_ublks;
    if (last_block_done(&st.ticket[kStUpdate], nblk)) {
        const int64_t b0 = c.f_ublk0;
        double a = 0.0, b = 0.0;
        for (int64_t i = threadIdx.x; i < (int64_t)nblk; i += kBlock) {
            a += __ldcg(partials + 2 * (b0 + i));
            b += __ldcg(partials + 2 * (b0 + i) + 1);
        }
        a = block_sum<kBlock>(a, sh);
        b = block_sum<kBlock>(b, sh);
        if (threadIdx.x == 0) {
            st.kinetic_energy = a;
            st.potential_energy = b;
            st.ticket[kStUpdate] = 0;
            ScenePersist &sp = k.sp[sc];
            sp.total_div_iter += st.div_iter;
            sp.total_incom_iter += st.incom_iter;
            sp.total_fbm_passes += st.fbm_passes;
            sp.max_dens_compression = fmax(sp.max_dens_compression, sp.compression);
            sp.steps += 1;
        }
    }
}

template <int DIM>
__global__ void __launch_bounds__(kBlock) k_update_bound(KConst k, tsph_set U, BoundBuf B,
                                                         const int *__restrict__ fstart) {
    pdl_entry();
    const int64_t pid = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (pid >= U.n) return;
    const int sc = k.b_user_scene[pid];
    const SceneConst &c = k.sc[sc];
    const SceneStep &st = k.ss[sc];
    if (pid == c.b_user) {
        // the density sweep of this step has run: BoundBuf::bb holds the
        // boundary-boundary sums of the boundary as gathered
        k.sp[sc].bb_valid = 1;
        k.sp[sc].bb_n = c.b_n;
    }
    const int64_t s = B.inv[pid];
    const float4 d = B.dens[s];
    U.W[pid] = d.x;
    U.sph_density[pid] = d.y;
    U.sph_compression[pid] = d.z;
    U.alpha_2[pid] = d.w;
    U.alpha[pid] = B.alpha[s];
    if (s - c.b_slot < st.b_in) {
        const int code = U.neighb_cell_seq[pid];
        U.neighb_in_cell_seq[pid] = (int)(s - st.b_shift) + fstart[c.cbase + code + 1];
    }
}

// ----------------------------------------------------------------------------- neighbours
__device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// Per particle: its neighbours with 0 < r < h in each set (FP32 q < 1, as the
// reference tests) and their order-independent hash, or -- cand != 0 -- the
// number of candidates the density sweep's scan visits in each grid (no hash).
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_neighbor_stats(KConst k, int bound, FluidBuf F, BoundBuf B,
                                                           int32_t *counts, uint64_t *hash, int cand) {
    pdl_entry();
    const int64_t s = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    const int64_t cap = bound ? B.cap : F.cap;
    if (s >= cap) return;
    const int sc = bound ? k.b_chunk_scene[s / kChunk] : k.f_chunk_scene[s / kChunk];
    const SceneConst &c = k.sc[sc];
    if (s - (bound ? c.b_slot : c.f_slot) >= (bound ? c.b_n : c.f_n)) return;
    const SceneStep &st = k.ss[sc];
    Geo g;
    g.load(c, k.R);
    const float4 pi = bound ? B.pos[s] : F.pos[s];
    bool ok;
    const long long code = cell_code<DIM>(pi, g, ok);
    int cf = 0, cb = 0;
    uint64_t hsum = 0;
    if (ok) {
        // the density sweep's visitor (it records the pairs every later sweep
        // walks): its skipped rows and cells must hold no pair with r < h
        visit_candidates_within<DIM>(F.start, g, pi, code, st.f_shift, 0, [&](int j) {
            const float4 pj = F.pos[j];
            const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (cand) {
                ++cf;
            } else if (r2 > 0.f && sqrtf(r2) * g.inv_h < 1.f) {
                ++cf;
                hsum += mix64((uint64_t)(uint32_t)F.perm[j]);
            }
        });
        visit_candidates_within<DIM>(B.start, g, pi, code, st.b_shift, 0, [&](int j) {
            const float4 pj = B.pos[j];
            const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (cand) {
                ++cb;
            } else if (r2 > 0.f && sqrtf(r2) * g.inv_h < 1.f) {
                ++cb;
                hsum += mix64((1ull << 32) | (uint64_t)(uint32_t)B.perm[j]);
            }
        });
    }
    const int pid = bound ? B.perm[s] : F.perm[s];
    counts[2 * pid] = cf;
    counts[2 * pid + 1] = cb;
    if (hash) hash[pid] = hsum;
}

// ----------------------------------------------------------------------------- launchers
void fork_side(tsph_ctx &c, cudaStream_t st) {
    if (!c.side) return;
    cudaEventRecord(c.ev_fork, st);
    cudaStreamWaitEvent(c.side, c.ev_fork, 0);
}

void join_side(tsph_ctx &c, cudaStream_t st) {
    if (!c.side) return;
    cudaEventRecord(c.ev_join, c.side);
    cudaStreamWaitEvent(st, c.ev_join, 0);
}

void launch_step_begin(tsph_ctx &c, cudaStream_t st) {
    cudaMemsetAsync(c.k.ss, 0, sizeof(SceneStep) * c.k.n_scenes, st);
    cudaMemsetAsync(c.k.dg, 0, sizeof(DevGlobal), st);
}

void launch_cfl(tsph_ctx &c, const tsph_set &f, cudaStream_t st) {
    int nb = blocks_for(f.n);
    if (nb < 1) nb = 1;
    if (nb > 4 * 152) nb = 4 * 152;
    c.launches += 1;
    if (c.k.dim == 3) TSPH_LAUNCH((k_cfl<3>), nb, kBlock, st, c.k, f.vel, f.n);
    else TSPH_LAUNCH((k_cfl<2>), nb, kBlock, st, c.k, f.vel, f.n);
}

void launch_grid_build(tsph_ctx &c, const tsph_set &f, const tsph_set &b, cudaStream_t st, bool with_cfl) {
    const int64_t nn = c.k.total_nodes;
    // the boundary set's encode, scatter and gather run on the side stream,
    // beside the fluid's; the scans cover both grids in one launch
    cudaStream_t sd = c.side ? c.side : st;
    c.launches += (f.n > 0) + (b.n > 0) + 2 + (f.n > 0) + (b.n > 0) + 2;
    fork_side(c, st);
    if (with_cfl) launch_cfl(c, f, sd);  // nothing before the first solve reads dt
    cudaMemsetAsync(c.B.count, 0, sizeof(int) * nn, sd);
    if (b.n > 0) {
        if (c.k.dim == 3) TSPH_LAUNCH((k_encode<3>), blocks_for(b.n), kBlock, sd, c.k, b, 1, c.B.count, c.B.slot);
        else TSPH_LAUNCH((k_encode<2>), blocks_for(b.n), kBlock, sd, c.k, b, 1, c.B.count, c.B.slot);
    }
    cudaMemsetAsync(c.F.count, 0, sizeof(int) * nn, st);
    if (f.n > 0) {
        if (c.k.dim == 3) TSPH_LAUNCH((k_encode<3>), blocks_for(f.n), kBlock, st, c.k, f, 0, c.F.count, c.F.slot);
        else TSPH_LAUNCH((k_encode<2>), blocks_for(f.n), kBlock, st, c.k, f, 0, c.F.count, c.F.slot);
    }
    join_side(c, st);
    ScanArgs sa;
    sa.count[0] = c.F.count; sa.count[1] = c.B.count;
    sa.start[0] = c.F.start; sa.start[1] = c.B.start;
    sa.blocks[0] = c.S.scan_blocks; sa.blocks[1] = c.S.scan_blocks + c.S.scan_len / 2;
    sa.n = nn;
    const int nblk = (int)((nn + kScanTile - 1) / kScanTile);
    TSPH_LAUNCH((k_scan_reduce), dim3(nblk, 2), kScanThreads, st, sa, nblk, c.k.dg->ticket + kGtScanF);
    TSPH_LAUNCH((k_scan_down), dim3(nblk, 2), kScanThreads, st, sa, nblk, c.k, c.k.dg->ticket + kGtScanDone);
    fork_side(c, st);
    if (b.n > 0) TSPH_LAUNCH((k_scatter), blocks_for(b.n), kBlock, sd, c.k, 1, b.n, b.neighb_cell_seq, c.B.slot, c.B.start, c.B.perm_u);
    if (f.n > 0) TSPH_LAUNCH((k_scatter), blocks_for(f.n), kBlock, st, c.k, 0, f.n, f.neighb_cell_seq, c.F.slot, c.F.start, c.F.perm_u);
    // each set's gather orders its cells by particle id as it copies (a
    // particle's slot is its rank among its cell's ids)
    if (c.k.dim == 3) {
        TSPH_LAUNCH((k_gather_bound<3>), blocks_for(c.B.cap), kBlock, sd, c.k, b, c.B);
        TSPH_LAUNCH((k_gather_fluid<3>), blocks_for(c.F.cap), kBlock, st, c.k, f, c.F);
    } else {
        TSPH_LAUNCH((k_gather_bound<2>), blocks_for(c.B.cap), kBlock, sd, c.k, b, c.B);
        TSPH_LAUNCH((k_gather_fluid<2>), blocks_for(c.F.cap), kBlock, st, c.k, f, c.F);
    }
    join_side(c, st);
}

void launch_unsort(tsph_ctx &c, const tsph_set &f, const tsph_set &b, cudaStream_t st) {
    const int fbm = c.p.fbm_enabled ? 1 : 0;
    const int st_on = c.st_on;
    // boundary: over the caller's count (the kernel returns past it); one block at least
    const int nbb = b.n > 0 ? blocks_for(b.n) : 1;
    c.launches += 2;
    cudaStream_t sd = c.side ? c.side : st;
    fork_side(c, st);
    if (c.k.dim == 3) {
        TSPH_LAUNCH((k_update_bound<3>), nbb, kBlock, sd, c.k, b, c.B, c.F.start);
        TSPH_LAUNCH((k_update_fluid<3>), (int)c.k.f_ublocks, kBlock, st, c.k, f, c.F, c.B.start, c.S.partials, fbm, st_on);
    } else {
        TSPH_LAUNCH((k_update_bound<2>), nbb, kBlock, sd, c.k, b, c.B, c.F.start);
        TSPH_LAUNCH((k_update_fluid<2>), (int)c.k.f_ublocks, kBlock, st, c.k, f, c.F, c.B.start, c.S.partials, fbm, st_on);
    }
    join_side(c, st);
}

void launch_neighbor_stats(tsph_ctx &c, int32_t *fc, uint64_t *fh, int32_t *bc, uint64_t *bh, int cand,
                           cudaStream_t st) {
    if (c.k.dim == 3) {
        k_neighbor_stats<3><<<blocks_for(c.F.cap), kBlock, 0, st>>>(c.k, 0, c.F, c.B, fc, fh, cand);
        k_neighbor_stats<3><<<blocks_for(c.B.cap), kBlock, 0, st>>>(c.k, 1, c.F, c.B, bc, bh, cand);
    } else {
        k_neighbor_stats<2><<<blocks_for(c.F.cap), kBlock, 0, st>>>(c.k, 0, c.F, c.B, fc, fh, cand);
        k_neighbor_stats<2><<<blocks_for(c.B.cap), kBlock, 0, st>>>(c.k, 1, c.F, c.B, bc, bh, cand);
    }
}

}  // namespace tsph
