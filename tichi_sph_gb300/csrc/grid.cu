// Cell grid build (counting sort) and the gather / scatter between the caller's
// particle order and the cell-sorted working order.
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
// cfl_condition, sph.py:41-47: dt = part_size / cs, lowered to
// part_size / |v| * cfl_factor for |v| > 1e-4.  part_size / v * cfl is monotone
// in v, so the minimum over particles is attained at max |v|.
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_cfl(KConst k, const float *__restrict__ vel, int64_t n,
                                                DevStep *ds, DevPersist *dp) {
    float vmax = 0.f;
    for (int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x; i < n; i += (int64_t)gridDim.x * kBlock) {
        float s = 0.f;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            float v = vel[i * DIM + d];
            s += v * v;
        }
        float vn = sqrtf(s);
        if (vn > 1e-4f) vmax = fmaxf(vmax, vn);  // NaN norms fail the test, as in the reference
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_down_sync(0xffffffffu, vmax, o));
    if ((threadIdx.x & 31) == 0 && vmax > 0.f) atomicMax(&ds->vmax_bits, __float_as_uint(vmax));
    if (last_block_done(&ds->ticket[0])) {
        if (threadIdx.x == 0) {
            float dt = __fdiv_rn(k.part_size, (float)k.cs);
            float vm = __uint_as_float(atomicAdd(&ds->vmax_bits, 0u));
            if (vm > 1e-4f) dt = fminf(dt, __fmul_rn(__fdiv_rn(k.part_size, vm), k.cfl));
            dp->dt = dt;
            dp->time_count += (double)dt;
            ds->ticket[0] = 0;
        }
    }
}

// ----------------------------------------------------------------------------- encode
// Ngrid.encode, sph_obj.py:300-306: structured cell, linear code, count.  A
// particle without a valid code gets a slot in the tail (after all in-grid ones).
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_encode(KConst k, tsph_set U, int *__restrict__ count,
                                                   int *__restrict__ slot, int *tail, int *status) {
    const int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (i >= U.n) return;
    float4 p = make_float4(U.pos[i * DIM], U.pos[i * DIM + 1], DIM == 3 ? U.pos[i * DIM + 2] : 0.f, 0.f);
    bool ok;
    long long code = cell_code<DIM>(p, k, ok);
    const float c[3] = {p.x, p.y, p.z};
#pragma unroll
    for (int d = 0; d < DIM; ++d)
        U.neighb_cell_structured_seq[i * DIM + d] = ok ? (int)floorf(__fdiv_rn(c[d] - k.lb[d], k.h)) : 0;
    U.neighb_cell_seq[i] = (int)code;
    int s;
    if (ok && code > 0 && code < k.node_num) {
        s = atomicAdd(count + code, 1);
    } else {
        s = -1 - atomicAdd(tail, 1);
        atomicOr(status, ok ? TSPH_ST_OUTSIDE_GRID : (TSPH_ST_NONFINITE_POS | TSPH_ST_OUTSIDE_GRID));
    }
    slot[i] = s;
}

// ----------------------------------------------------------------------------- scan
// Exclusive scan of the cell counts: 4096 cells per block, then a single-block
// scan of the block totals, then the add.  blockIdx.y selects the fluid (0) or
// boundary (1) grid.
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

__global__ void __launch_bounds__(kScanThreads) k_scan_local(ScanArgs a) {
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
    int run = block_excl_scan(sum, sh, total);
#pragma unroll
    for (int t = 0; t < kScanItems; ++t) {
        if (base + t < a.n) a.start[g][base + t] = run;
        run += v[t];
    }
    if (threadIdx.x == 0) a.blocks[g][blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_blocks(ScanArgs a, int nblocks) {
    __shared__ int sh[33];
    const int g = blockIdx.y;
    int carry = 0;
    for (int base = 0; base < nblocks; base += kScanTile) {
        int v[kScanItems];
        int sum = 0;
        const int i0 = base + threadIdx.x * kScanItems;
#pragma unroll
        for (int t = 0; t < kScanItems; ++t) {
            v[t] = (i0 + t < nblocks) ? a.blocks[g][i0 + t] : 0;
            sum += v[t];
        }
        int total;
        int run = block_excl_scan(sum, sh, total) + carry;
#pragma unroll
        for (int t = 0; t < kScanItems; ++t) {
            if (i0 + t < nblocks) a.blocks[g][i0 + t] = run;
            run += v[t];
        }
        carry += total;
    }
    if (threadIdx.x == 0) a.blocks[g][nblocks] = carry;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_add(ScanArgs a, int nblocks) {
    const int g = blockIdx.y;
    const int add = a.blocks[g][blockIdx.x];
    const int64_t base = blockIdx.x * (int64_t)kScanTile;
    for (int t = threadIdx.x; t < kScanTile; t += kScanThreads)
        if (base + t < a.n) a.start[g][base + t] += add;
    if (blockIdx.x == 0 && threadIdx.x == 0) a.start[g][a.n] = a.blocks[g][nblocks];
}

// ----------------------------------------------------------------------------- scatter
struct ScatterArgs {
    const int *code[2];
    const int *slot[2];
    const int *start[2];
    int *perm[2];
    int64_t n[2];
    long long node_num;
};

__global__ void __launch_bounds__(kBlock) k_scatter(ScatterArgs a) {
    const int g = blockIdx.y;
    const int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (i >= a.n[g]) return;
    const int sl = a.slot[g][i];
    int s;
    if (sl >= 0) s = a.start[g][a.code[g][i]] + sl;
    else s = a.start[g][a.node_num] + (-1 - sl);
    a.perm[g][s] = (int)i;
}

// Orders each cell's particles by id (insertion sort; cells hold ~2^dim..30).
// Tail particles (no valid cell) are ordered too, by one thread per set.
struct CellSortArgs {
    const int *start[2];
    int *perm[2];
    int64_t n[2];
    long long node_num;
};

__device__ __forceinline__ void insertion_sort(int *p, int beg, int end) {
    for (int a = beg + 1; a < end; ++a) {
        int v = p[a];
        int b = a - 1;
        while (b >= beg && p[b] > v) {
            p[b + 1] = p[b];
            --b;
        }
        p[b + 1] = v;
    }
}

__global__ void __launch_bounds__(kBlock) k_cell_sort(CellSortArgs a) {
    const int g = blockIdx.y;
    const long long c = blockIdx.x * (long long)kBlock + threadIdx.x;
    if (c < a.node_num) {
        const int beg = a.start[g][c], end = a.start[g][c + 1];
        if (end - beg > 1) insertion_sort(a.perm[g], beg, end);
    } else if (c == a.node_num) {
        insertion_sort(a.perm[g], a.start[g][a.node_num], (int)a.n[g]);
    }
}

// ----------------------------------------------------------------------------- gather
// Copies the caller-order state into the sorted working arrays; v_adv = vel
// (SPH_vel_2_vel_adv, sph.py:253-256).  X / psi0 follow the solver aliases,
// sph_obj.py:65-73.
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_gather_fluid(KConst k, tsph_set U, FluidBuf F) {
    const int64_t s = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (s >= U.n) return;
    const int pid = F.perm[s];
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
    const int64_t s = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (s >= U.n) return;
    const int pid = B.perm[s];
    B.inv[pid] = (int)s;
    const float *p = U.pos + (int64_t)pid * DIM;
    const float *va = U.vel_adv + (int64_t)pid * DIM;
    const float m = U.mass[pid], V = U.rest_volume[pid];
    B.pos[s] = make_float4(p[0], p[1], DIM == 3 ? p[2] : 0.f, k.vfsph ? V : m);
    B.mv[s] = make_float2(m, V);
    B.vadv[s] = make_float4(va[0], va[1], DIM == 3 ? va[2] : 0.f, 0.f);
    B.kappa[s] = U.psi_adv[pid];  // divided by alpha once alpha is known
}

// ----------------------------------------------------------------------------- unsort
// Writes the step's results back in caller order, fused with SPH_update_volume_frac,
// SPH_update_mass, SPH_update_pos and SPH_update_energy (sph.py:265-286, 375-379).
// Energies: per-particle FP32 terms, FP64 block sums, fixed-order final sum.
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_unsort_fluid(KConst k, tsph_set U, FluidBuf F,
                                                         const int *__restrict__ bstart, DevStep *ds,
                                                         DevPersist *dp, double *partials,
                                                         int fbm, int st_on) {
    __shared__ double sh[kBlock / 32];
    const int64_t pid = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    double ke = 0.0, pe = 0.0;
    if (pid < U.n) {
        const int s = F.inv[pid];
        const int cur = ds->cur;
        const float dt = dp->dt;
        const float4 v = F.vadv[cur * F.cap + s];
        const float4 p = F.pos[s];
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
            rho0 += k.rho_phase[q] * vf;
        }
        const float m = rho0 * V;
        const float np[3] = {p.x + v.x * dt, p.y + v.y * dt, p.z + v.z * dt};
        const float vv[3] = {v.x, v.y, v.z};
        const float4 acc = F.acc[s];
        const float aa[3] = {acc.x, acc.y, acc.z};
        const float4 a1 = F.a1[s];
        const float a1v[3] = {a1.x, a1.y, a1.z};
        const float4 nr = F.normal[s];
        const float nrv[3] = {nr.x, nr.y, nr.z};
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            U.pos[pid * DIM + d] = np[d];
            U.vel[pid * DIM + d] = vv[d];
            U.vel_adv[pid * DIM + d] = vv[d];
            U.acce_adv[pid * DIM + d] = aa[d];
            U.alpha_1[pid * DIM + d] = a1v[d];
            if (st_on) U.normal[pid * DIM + d] = nrv[d];
        }
        if (fbm) {
            const float4 fa = F.facc[s];
            const float fav[3] = {fa.x, fa.y, fa.z};
#pragma unroll
            for (int d = 0; d < DIM; ++d) U.acce[pid * DIM + d] = fav[d];
            for (int q = 0; q < k.P; ++q) {
                const float4 dv = F.drift[q * F.cap + s];
                const float dvv[3] = {dv.x, dv.y, dv.z};
#pragma unroll
                for (int d = 0; d < DIM; ++d) U.drift_vel[(pid * k.P + q) * DIM + d] = dvv[d];
            }
            U.fbm_zeta[pid] = F.zeta[s];
        }
        U.flag[pid] = flagged;
        U.mass[pid] = m;
        U.rest_density[pid] = rho0;
        U.W[pid] = F.W[s];
        U.sph_density[pid] = F.rho[s];
        U.sph_compression[pid] = F.comp[s];
        U.psi_adv[pid] = F.psiadv[s];
        U.alpha[pid] = F.mpsi[s].w;
        U.alpha_2[pid] = F.a2[s];
        const int code = U.neighb_cell_seq[pid];
        if (code > 0 && code < k.node_num && s < F.start[k.node_num]) U.neighb_in_cell_seq[pid] = s + bstart[code];
        float v2 = 0.f;
#pragma unroll
        for (int d = 0; d < DIM; ++d) v2 += vv[d] * vv[d];
        ke = (double)(0.5f * m * v2);
        pe = (double)(-m * k.g[1] * (np[1] - k.lb[1]));
    }
    double bke = block_sum<kBlock>(ke, sh);
    double bpe = block_sum<kBlock>(pe, sh);
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = bke;
        partials[2 * blockIdx.x + 1] = bpe;
    }
    if (last_block_done(&ds->ticket[1])) {
        double a = 0.0, b = 0.0;
        for (int i = threadIdx.x; i < (int)gridDim.x; i += kBlock) {
            a += __ldcg(partials + 2 * i);
            b += __ldcg(partials + 2 * i + 1);
        }
        a = block_sum<kBlock>(a, sh);
        b = block_sum<kBlock>(b, sh);
        if (threadIdx.x == 0) {
            ds->kinetic_energy = a;
            ds->potential_energy = b;
            ds->ticket[1] = 0;
            dp->total_div_iter += ds->div_iter;
            dp->total_incom_iter += ds->incom_iter;
            dp->total_fbm_passes += ds->fbm_passes;
            dp->max_dens_compression = fmax(dp->max_dens_compression, dp->compression);
        }
    }
}

template <int DIM>
__global__ void __launch_bounds__(kBlock) k_unsort_bound(KConst k, tsph_set U, BoundBuf B,
                                                         const int *__restrict__ fstart) {
    const int64_t pid = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (pid >= U.n) return;
    const int s = B.inv[pid];
    U.W[pid] = B.W[s];
    U.sph_density[pid] = B.rho[s];
    U.sph_compression[pid] = B.comp[s];
    U.alpha_2[pid] = B.a2[s];
    U.alpha[pid] = B.alpha[s];
    const int code = U.neighb_cell_seq[pid];
    if (code > 0 && code < k.node_num && s < B.start[k.node_num]) U.neighb_in_cell_seq[pid] = s + fstart[code + 1];
}

// ----------------------------------------------------------------------------- neighbours
__device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

template <int DIM>
__global__ void __launch_bounds__(kBlock) k_neighbor_stats(KConst k, const float4 *__restrict__ pos,
                                                           const int *__restrict__ perm, int64_t n,
                                                           FluidBuf F, BoundBuf B, int32_t *counts,
                                                           uint64_t *hash) {
    const int64_t s = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (s >= n) return;
    const float4 pi = pos[s];
    bool ok;
    const long long code = cell_code<DIM>(pi, k, ok);
    int cf = 0, cb = 0;
    uint64_t hsum = 0;
    if (ok) {
        visit_candidates<DIM>(F.start, k, code, [&](int j) {
            const float4 pj = F.pos[j];
            const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (r2 > 0.f && sqrtf(r2) * k.inv_h < 1.f) {
                ++cf;
                hsum += mix64((uint64_t)(uint32_t)F.perm[j]);
            }
        });
        visit_candidates<DIM>(B.start, k, code, [&](int j) {
            const float4 pj = B.pos[j];
            const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (r2 > 0.f && sqrtf(r2) * k.inv_h < 1.f) {
                ++cb;
                hsum += mix64((1ull << 32) | (uint64_t)(uint32_t)B.perm[j]);
            }
        });
    }
    const int pid = perm[s];
    counts[2 * pid] = cf;
    counts[2 * pid + 1] = cb;
    hash[pid] = hsum;
}

// ----------------------------------------------------------------------------- launchers
void launch_step_begin(tsph_ctx &c, cudaStream_t st) {
    cudaMemsetAsync(c.ds, 0, sizeof(DevStep), st);
}

void launch_cfl(tsph_ctx &c, const tsph_set &f, cudaStream_t st) {
    int nb = blocks_for(f.n);
    if (nb < 1) nb = 1;
    if (nb > 4 * 152) nb = 4 * 152;
    c.launches += 1;
    if (c.k.dim == 3) k_cfl<3><<<nb, kBlock, 0, st>>>(c.k, f.vel, f.n, c.ds, c.dp);
    else k_cfl<2><<<nb, kBlock, 0, st>>>(c.k, f.vel, f.n, c.ds, c.dp);
}

void launch_grid_build(tsph_ctx &c, const tsph_set &f, const tsph_set &b, cudaStream_t st) {
    const int64_t nn = c.k.node_num;
    cudaMemsetAsync(c.F.count, 0, sizeof(int) * nn, st);
    cudaMemsetAsync(c.B.count, 0, sizeof(int) * nn, st);
    c.launches += (f.n > 0) + (b.n > 0) + 3 + 1 + (f.n > 0) + (b.n > 0) + ((f.n > 0 || b.n > 0) ? 1 : 0);
    if (f.n > 0) {
        if (c.k.dim == 3) k_encode<3><<<blocks_for(f.n), kBlock, 0, st>>>(c.k, f, c.F.count, c.F.slot, &c.ds->f_tail, &c.ds->status);
        else k_encode<2><<<blocks_for(f.n), kBlock, 0, st>>>(c.k, f, c.F.count, c.F.slot, &c.ds->f_tail, &c.ds->status);
    }
    if (b.n > 0) {
        if (c.k.dim == 3) k_encode<3><<<blocks_for(b.n), kBlock, 0, st>>>(c.k, b, c.B.count, c.B.slot, &c.ds->b_tail, &c.ds->status);
        else k_encode<2><<<blocks_for(b.n), kBlock, 0, st>>>(c.k, b, c.B.count, c.B.slot, &c.ds->b_tail, &c.ds->status);
    }
    ScanArgs sa;
    sa.count[0] = c.F.count; sa.count[1] = c.B.count;
    sa.start[0] = c.F.start; sa.start[1] = c.B.start;
    sa.blocks[0] = c.S.scan_blocks; sa.blocks[1] = c.S.scan_blocks + c.S.scan_len / 2;
    sa.n = nn;
    const int nblk = (int)((nn + kScanTile - 1) / kScanTile);
    k_scan_local<<<dim3(nblk, 2), kScanThreads, 0, st>>>(sa);
    k_scan_blocks<<<dim3(1, 2), kScanThreads, 0, st>>>(sa, nblk);
    k_scan_add<<<dim3(nblk, 2), kScanThreads, 0, st>>>(sa, nblk);
    const int64_t nmax = f.n > b.n ? f.n : b.n;
    if (nmax > 0) {
        ScatterArgs sc;
        sc.code[0] = f.neighb_cell_seq; sc.code[1] = b.neighb_cell_seq;
        sc.slot[0] = c.F.slot; sc.slot[1] = c.B.slot;
        sc.start[0] = c.F.start; sc.start[1] = c.B.start;
        sc.perm[0] = c.F.perm; sc.perm[1] = c.B.perm;
        sc.n[0] = f.n; sc.n[1] = b.n;
        sc.node_num = nn;
        k_scatter<<<dim3(blocks_for(nmax), 2), kBlock, 0, st>>>(sc);
    }
    CellSortArgs cs;
    cs.start[0] = c.F.start; cs.start[1] = c.B.start;
    cs.perm[0] = c.F.perm; cs.perm[1] = c.B.perm;
    cs.n[0] = f.n; cs.n[1] = b.n;
    cs.node_num = nn;
    k_cell_sort<<<dim3(blocks_for(nn + 1), 2), kBlock, 0, st>>>(cs);
    if (f.n > 0) {
        if (c.k.dim == 3) k_gather_fluid<3><<<blocks_for(f.n), kBlock, 0, st>>>(c.k, f, c.F);
        else k_gather_fluid<2><<<blocks_for(f.n), kBlock, 0, st>>>(c.k, f, c.F);
    }
    if (b.n > 0) {
        if (c.k.dim == 3) k_gather_bound<3><<<blocks_for(b.n), kBlock, 0, st>>>(c.k, b, c.B);
        else k_gather_bound<2><<<blocks_for(b.n), kBlock, 0, st>>>(c.k, b, c.B);
    }
}

void launch_unsort(tsph_ctx &c, const tsph_set &f, const tsph_set &b, cudaStream_t st) {
    const int fbm = c.p.fbm_enabled ? 1 : 0;
    const int st_on = c.k.gamma != 0.f ? 1 : 0;
    int nb = blocks_for(f.n);
    if (nb < 1) nb = 1;
    c.launches += 1 + (b.n > 0);
    if (c.k.dim == 3) k_unsort_fluid<3><<<nb, kBlock, 0, st>>>(c.k, f, c.F, c.B.start, c.ds, c.dp, c.S.partials, fbm, st_on);
    else k_unsort_fluid<2><<<nb, kBlock, 0, st>>>(c.k, f, c.F, c.B.start, c.ds, c.dp, c.S.partials, fbm, st_on);
    if (b.n > 0) {
        if (c.k.dim == 3) k_unsort_bound<3><<<blocks_for(b.n), kBlock, 0, st>>>(c.k, b, c.B, c.F.start);
        else k_unsort_bound<2><<<blocks_for(b.n), kBlock, 0, st>>>(c.k, b, c.B, c.F.start);
    }
}

void launch_neighbor_stats(tsph_ctx &c, int64_t nf, int64_t nb, int32_t *fc, uint64_t *fh, int32_t *bc,
                           uint64_t *bh, cudaStream_t st) {
    if (nf > 0) {
        if (c.k.dim == 3) k_neighbor_stats<3><<<blocks_for(nf), kBlock, 0, st>>>(c.k, c.F.pos, c.F.perm, nf, c.F, c.B, fc, fh);
        else k_neighbor_stats<2><<<blocks_for(nf), kBlock, 0, st>>>(c.k, c.F.pos, c.F.perm, nf, c.F, c.B, fc, fh);
    }
    if (nb > 0) {
        if (c.k.dim == 3) k_neighbor_stats<3><<<blocks_for(nb), kBlock, 0, st>>>(c.k, c.B.pos, c.B.perm, nb, c.F, c.B, bc, bh);
        else k_neighbor_stats<2><<<blocks_for(nb), kBlock, 0, st>>>(c.k, c.B.pos, c.B.perm, nb, c.F, c.B, bc, bh);
    }
}

}  // namespace tsph
