// Fluid density sweep that allocates nothing: tsph_fluid_density_noalloc.
//
// Who needs it: callers that must not allocate device memory at the point they
// call in -- plugin and real-time hosts that pre-plan every byte of device
// memory and forbid allocations on their worker threads, and embedders whose
// own allocator owns the device (a cudaMalloc behind its back breaks its
// accounting or fails for want of memory it has already reserved).  They cannot hold a tsph_ctx (tsph_create allocates), so this
// entry point computes the fluid's SPH_prepare_attr sums (W, sph_density,
// sph_compression over fluid and boundary neighbours; sph.py:50-64, called as
// main.py:188-189) from caller-owned inputs into caller-owned outputs.
//
// Its working memory (two cell grids and two particle permutations) is one
// file-scope device array, g_noalloc_scratch, of fixed size: at most
// TSPH_NOALLOC_MAX_CELLS cells and TSPH_NOALLOC_MAX_PARTICLES particles per set.
// Every GPU that loads this library holds that array until the process exits.
// All calls share it and it keeps the previous call's contents, so each call
// clears what must start at zero, and calls that overlap on the GPU (different
// streams, or different host threads) race on it: serialise them.
//
// Host code cannot use the array's name as a device address (in host code the
// symbol is a host-side stand-in).  The first call on each device therefore
// looks the address up with cudaGetSymbolAddress while that device is current,
// checks the result and caches it; make that first call before any stream
// capture begins, since the lookup is not a capturable operation.  The cached
// address belongs to the device's primary context as it was at that first
// call: a cudaDeviceReset afterwards, or calls from a context other than the
// primary one, are not supported.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdio>

#include "ctx.h"

namespace tsph {
void set_last_error_text(const char *msg);
}

using namespace tsph;

namespace {

constexpr int64_t kMaxCells = TSPH_NOALLOC_MAX_CELLS;
constexpr int64_t kMaxParts = TSPH_NOALLOC_MAX_PARTICLES;

// Scratch layout, in ints: per set g in {fluid, boundary}
//   count[g][kMaxCells], start[g][kMaxCells + 1], slot[g][kMaxParts], perm[g][kMaxParts],
// then tail[2] (particles without a valid cell).
constexpr int64_t kOffCount = 0;
constexpr int64_t kOffStart = kOffCount + 2 * kMaxCells;
constexpr int64_t kOffSlot = kOffStart + 2 * (kMaxCells + 1);
constexpr int64_t kOffPerm = kOffSlot + 2 * kMaxParts;
constexpr int64_t kOffTail = kOffPerm + 2 * kMaxParts;
constexpr int64_t kScratchInts = kOffTail + 8;

static __device__ __align__(256) int g_noalloc_scratch[kScratchInts];

constexpr int kMaxDevices = 64;
std::atomic<int *> g_scratch_ptr[kMaxDevices];

struct Grids {
    int *count[2], *start[2], *slot[2], *perm[2], *tail;
};

Grids carve(int *base) {
    Grids g;
    for (int s = 0; s < 2; ++s) {
        g.count[s] = base + kOffCount + s * kMaxCells;
        g.start[s] = base + kOffStart + s * (kMaxCells + 1);
        g.slot[s] = base + kOffSlot + s * kMaxParts;
        g.perm[s] = base + kOffPerm + s * kMaxParts;
    }
    g.tail = base + kOffTail;
    return g;
}

struct SetIn {
    const float *pos, *mass, *rest_volume;
    int64_t n;
};

template <int DIM>
__device__ __forceinline__ float4 load_pos(const float *pos, int64_t i) {
    return make_float4(pos[i * DIM], pos[i * DIM + 1], DIM == 3 ? pos[i * DIM + 2] : 0.f, 0.f);
}

template <int DIM>
__global__ void k_na_encode(Geo k, SetIn in, int *count, int *slot, int *tail) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= in.n) return;
    bool ok;
    const long long code = cell_code<DIM>(load_pos<DIM>(in.pos, i), k, ok);
    slot[i] = (ok && code > 0 && code < k.node_num) ? atomicAdd(count + code, 1) : -1 - atomicAdd(tail, 1);
}

// Exclusive scan of up to kMaxCells counts by one block of 1024 threads: each
// thread owns a contiguous chunk, chunk sums are scanned across the block.
// start[n] receives the total.
__global__ void __launch_bounds__(1024) k_na_scan(const int *count, int *start, int64_t n) {
    __shared__ int warp_tot[32];
    const int64_t chunk = (n + 1023) / 1024;
    const int64_t lo = threadIdx.x * chunk;
    const int64_t hi = lo + chunk < n ? lo + chunk : n;
    int sum = 0;
    for (int64_t i = lo; i < hi; ++i) sum += count[i];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = sum;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
        const int t = warp_tot[lane];
        int u = t;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, u, o);
            if (lane >= o) u += y;
        }
        warp_tot[lane] = u - t;
        if (lane == 31) start[n] = u;
    }
    __syncthreads();
    int run = warp_tot[w] + x - sum;
    for (int64_t i = lo; i < hi; ++i) {
        start[i] = run;
        run += count[i];
    }
}

template <int DIM>
__global__ void k_na_scatter(Geo k, SetIn in, const int *slot, const int *start, int *perm) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= in.n) return;
    const int sl = slot[i];
    int64_t s;
    if (sl >= 0) {
        bool ok;
        const long long code = cell_code<DIM>(load_pos<DIM>(in.pos, i), k, ok);
        s = start[code] + sl;
    } else {
        s = start[k.node_num] + (-1 - sl);
    }
    perm[s] = (int)i;
}

// Orders each cell's slots by particle id (and the tail), as the step's grid does.
__global__ void k_na_sort(const int *start0, int *perm0, int64_t n0, const int *start1, int *perm1, int64_t n1,
                          int64_t node_num) {
    const int g = blockIdx.y;
    const int *start = g ? start1 : start0;
    int *perm = g ? perm1 : perm0;
    const int64_t n = g ? n1 : n0;
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int beg, end;
    if (c < node_num) {
        beg = start[c];
        end = start[c + 1];
    } else if (c == node_num) {
        beg = start[node_num];
        end = (int)n;
    } else {
        return;
    }
    for (int a = beg + 1; a < end; ++a) {
        const int v = perm[a];
        int b = a - 1;
        while (b >= beg && perm[b] > v) {
            perm[b + 1] = perm[b];
            --b;
        }
        perm[b + 1] = v;
    }
}

// W, sph_density, sph_compression of every fluid particle over its fluid and
// boundary candidates (SPH_prepare_attr (f,f) then (f,b), sph.py:50-64), with
// the same candidate order and arithmetic as the step's density sweep.
template <int DIM>
__global__ void k_na_density(Geo k, SetIn f, SetIn b, const int *fstart, const int *fperm, const int *bstart,
                             const int *bperm, float *W, float *rho, float *comp) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= f.n) return;
    const float4 pi = load_pos<DIM>(f.pos, i);
    bool ok;
    const long long code = cell_code<DIM>(pi, k, ok);
    float wsum = 0.f, rh = 0.f, cp = 0.f;
    if (ok) {
        visit_candidates<DIM>(fstart, k, code, 0, 0, [&](int j) {
            const int pid = fperm[j];
            const float4 pj = load_pos<DIM>(f.pos, pid);
            const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (r2 < k.h2) {
                const float w = kw(sqrtf(r2) * k.inv_h) * k.sig;
                wsum += w;
                rh += w * f.mass[pid];
                cp += w * f.rest_volume[pid];
            }
        });
        visit_candidates<DIM>(bstart, k, code, 0, 0, [&](int j) {
            const int pid = bperm[j];
            const float4 pj = load_pos<DIM>(b.pos, pid);
            const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (r2 < k.h2) {
                const float w = kw(sqrtf(r2) * k.inv_h) * k.sig;
                wsum += w;
                rh += w * b.mass[pid];
                cp += w * b.rest_volume[pid];
            }
        });
    }
    W[i] = wsum;
    rho[i] = rh;
    comp[i] = cp;
}

int na_fail(int code, const char *msg) {
    set_last_error_text(msg);
    return code;
}

int na_fail_cuda(cudaError_t e, const char *what) {
    char buf[256];
    std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    set_last_error_text(buf);
    return TSPH_ERR_CUDA;
}

}  // namespace

extern "C" int tsph_fluid_density_noalloc(const tsph_params *p, const float *fluid_pos, const float *fluid_mass,
                                          const float *fluid_rest_volume, int64_t n_fluid, const float *bound_pos,
                                          const float *bound_mass, const float *bound_rest_volume, int64_t n_bound,
                                          float *W, float *sph_density, float *sph_compression, void *stream) {
    if (!p) return na_fail(TSPH_ERR_INVALID, "tsph_fluid_density_noalloc: null params");
    if (p->dim != 2 && p->dim != 3) return na_fail(TSPH_ERR_INVALID, "tsph_fluid_density_noalloc: dim must be 2 or 3");
    if (!(p->kernel_h > 0.f)) return na_fail(TSPH_ERR_INVALID, "tsph_fluid_density_noalloc: kernel_h must be positive");
    if (p->neighb_range < 0 || p->neighb_range > 8)
        return na_fail(TSPH_ERR_INVALID, "tsph_fluid_density_noalloc: neighb_range out of range");
    if (p->node_num < 1) return na_fail(TSPH_ERR_INVALID, "tsph_fluid_density_noalloc: node_num must be >= 1");
    if (n_fluid < 0 || n_bound < 0) return na_fail(TSPH_ERR_INVALID, "tsph_fluid_density_noalloc: negative count");
    char msg[200];
    if (p->node_num > kMaxCells) {
        std::snprintf(msg, sizeof(msg),
                      "tsph_fluid_density_noalloc: %lld grid cells exceed its fixed scratch of %lld cells "
                      "(TSPH_NOALLOC_MAX_CELLS); use tsph_create / tsph_sph_step",
                      (long long)p->node_num, (long long)kMaxCells);
        return na_fail(TSPH_ERR_CAPACITY, msg);
    }
    if (n_fluid > kMaxParts || n_bound > kMaxParts) {
        std::snprintf(msg, sizeof(msg),
                      "tsph_fluid_density_noalloc: %lld fluid / %lld boundary particles exceed its fixed scratch of "
                      "%lld per set (TSPH_NOALLOC_MAX_PARTICLES); use tsph_create / tsph_sph_step",
                      (long long)n_fluid, (long long)n_bound, (long long)kMaxParts);
        return na_fail(TSPH_ERR_CAPACITY, msg);
    }
    if ((n_fluid > 0 && (!fluid_pos || !fluid_mass || !fluid_rest_volume || !W || !sph_density || !sph_compression)) ||
        (n_bound > 0 && (!bound_pos || !bound_mass || !bound_rest_volume)))
        return na_fail(TSPH_ERR_INVALID, "tsph_fluid_density_noalloc: null array");
    if (n_fluid == 0) return TSPH_OK;

    // an error left pending by an earlier call of the caller is not this call's:
    // take it off so that the check after the launches reports only these
    (void)cudaGetLastError();
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return na_fail_cuda(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return na_fail(TSPH_ERR_INVALID, "tsph_fluid_density_noalloc: device index too large");
    int *base = g_scratch_ptr[dev].load(std::memory_order_acquire);
    if (!base) {
        // once per device, with that device current
        e = cudaGetSymbolAddress((void **)&base, g_noalloc_scratch);
        if (e != cudaSuccess) return na_fail_cuda(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_scratch_ptr[dev].store(base, std::memory_order_release);
    }
    const Grids g = carve(base);

    Geo k = {};
    for (int d = 0; d < 3; ++d) k.lb[d] = d < p->dim ? p->lb[d] : 0.f;
    k.h = p->kernel_h;
    k.h2 = p->kernel_h2;
    k.inv_h = 1.f / p->kernel_h;
    k.sig = p->kernel_sig;
    k.sig_h = p->kernel_sig / p->kernel_h;
    k.node_num = p->node_num;
    k.nx = p->grid_size[0];
    k.nxny = (long long)p->grid_size[0] * (p->dim == 3 ? p->grid_size[1] : 1);
    k.cbase = 0;
    k.R = p->neighb_range;

    cudaStream_t st = (cudaStream_t)stream;
    const int64_t nn = p->node_num;
    // the scratch keeps the previous call's contents: clear the counters
    e = cudaMemsetAsync(g.count[0], 0, sizeof(int) * nn, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(g.count[1], 0, sizeof(int) * nn, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(g.tail, 0, sizeof(int) * 2, st);
    if (e != cudaSuccess) return na_fail_cuda(e, "tsph_fluid_density_noalloc: clearing the scratch counters");
    const SetIn fi = {fluid_pos, fluid_mass, fluid_rest_volume, n_fluid};
    const SetIn bi = {bound_pos, bound_mass, bound_rest_volume, n_bound};
    const int bs = 256;
    const int gf = (int)((n_fluid + bs - 1) / bs), gb = (int)((n_bound + bs - 1) / bs);
    const int gc = (int)((nn + 1 + bs - 1) / bs);
    if (p->dim == 3) {
        k_na_encode<3><<<gf, bs, 0, st>>>(k, fi, g.count[0], g.slot[0], g.tail);
        if (n_bound > 0) k_na_encode<3><<<gb, bs, 0, st>>>(k, bi, g.count[1], g.slot[1], g.tail + 1);
    } else {
        k_na_encode<2><<<gf, bs, 0, st>>>(k, fi, g.count[0], g.slot[0], g.tail);
        if (n_bound > 0) k_na_encode<2><<<gb, bs, 0, st>>>(k, bi, g.count[1], g.slot[1], g.tail + 1);
    }
    k_na_scan<<<1, 1024, 0, st>>>(g.count[0], g.start[0], nn);
    k_na_scan<<<1, 1024, 0, st>>>(g.count[1], g.start[1], nn);
    if (p->dim == 3) {
        k_na_scatter<3><<<gf, bs, 0, st>>>(k, fi, g.slot[0], g.start[0], g.perm[0]);
        if (n_bound > 0) k_na_scatter<3><<<gb, bs, 0, st>>>(k, bi, g.slot[1], g.start[1], g.perm[1]);
    } else {
        k_na_scatter<2><<<gf, bs, 0, st>>>(k, fi, g.slot[0], g.start[0], g.perm[0]);
        if (n_bound > 0) k_na_scatter<2><<<gb, bs, 0, st>>>(k, bi, g.slot[1], g.start[1], g.perm[1]);
    }
    k_na_sort<<<dim3(gc, 2), bs, 0, st>>>(g.start[0], g.perm[0], n_fluid, g.start[1], g.perm[1], n_bound, nn);
    if (p->dim == 3)
        k_na_density<3><<<gf, bs, 0, st>>>(k, fi, bi, g.start[0], g.perm[0], g.start[1], g.perm[1], W, sph_density,
                                           sph_compression);
    else
        k_na_density<2><<<gf, bs, 0, st>>>(k, fi, bi, g.start[0], g.perm[0], g.start[1], g.perm[1], W, sph_density,
                                           sph_compression);
    e = cudaGetLastError();
    if (e != cudaSuccess) return na_fail_cuda(e, "tsph_fluid_density_noalloc launch");
    return TSPH_OK;
}
