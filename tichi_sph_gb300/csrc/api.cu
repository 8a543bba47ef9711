// C ABI of the SPH hot path: context management and the per-substep schedule.
//
// The substep (run_step's body, main.py:348-352, around sph_step, main.py:175-256)
// is captured once into a CUDA graph per (particle counts, array pointers) and
// replayed.  Both data-dependent loops of the reference -- the two Jacobi solves
// (main.py:201-213, 222-234) and the volume-fraction pass loop (main.py:244-248)
// -- become device-side while nodes whose condition is set by the last block of
// the loop body, so a substep runs without any host round trip.  The host-driven
// mode (tsph_set_graph_mode(ctx, 0)) replays the same kernels with a
// device-to-host read of the loop condition per iteration, as the reference does.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "ctx.h"

using namespace tsph;

namespace {

thread_local char g_last_error[256] = "";

int fail_cuda(cudaError_t e, const char *what) {
    std::snprintf(g_last_error, sizeof(g_last_error), "%s: %s", what, cudaGetErrorString(e));
    return TSPH_ERR_CUDA;
}

int fail(int code, const char *what) {
    std::snprintf(g_last_error, sizeof(g_last_error), "%s", what);
    return code;
}

#define TSPH_CK(call)                                            \
    do {                                                         \
        cudaError_t e_ = (call);                                 \
        if (e_ != cudaSuccess) return fail_cuda(e_, #call);      \
    } while (0)

struct Alloc {
    std::vector<void *> ptrs;
    cudaError_t err = cudaSuccess;
    template <class T>
    T *get(int64_t n) {
        if (n < 1) n = 1;
        void *p = nullptr;
        cudaError_t e = cudaMalloc(&p, sizeof(T) * (size_t)n);
        if (e != cudaSuccess) {
            err = e;
            return nullptr;
        }
        cudaMemset(p, 0, sizeof(T) * (size_t)n);
        ptrs.push_back(p);
        return (T *)p;
    }
};

struct CtxExtra {
    Alloc alloc;
    cudaStream_t cap_stream = nullptr;
    cudaStream_t body_stream = nullptr;
};

CtxExtra *extra(tsph_ctx *c);

__global__ void k_set_state(DevPersist *dp, double time_count, float dt, double compression) {
    dp->time_count = time_count;
    dp->dt = dt;
    dp->compression = compression;
}

// Solve with no fluid particle: the reference still runs min(iter_min, iter_max+1)
// empty iterations and compression becomes 0/0 = NaN (sph.py:226).
__global__ void k_solve_empty(KConst k, DevStep *ds, DevPersist *dp, int kind) {
    int it = 0;
    bool any = false;
    while (it < k.iter_min) {
        any = true;
        ++it;
        if (it > k.iter_max) break;
    }
    if (any) dp->compression = __longlong_as_double(0x7ff8000000000000ll);
    if (kind == kSolveDiv) ds->div_iter = it;
    else ds->incom_iter = it;
}

int solve(tsph_ctx &c, int64_t nf, int kind, cudaStream_t st, bool graph) {
    if (nf <= 0) {
        k_solve_empty<<<1, 1, 0, st>>>(c.k, c.ds, c.dp, kind);
        c.launches += 1;
        return TSPH_OK;
    }
    if (!graph) {
        launch_solve_begin(c, kind, 0, 0, st);
        for (;;) {
            TSPH_CK(cudaMemcpyAsync(&c.host_ds->cond, &c.ds->cond, sizeof(int), cudaMemcpyDeviceToHost, st));
            TSPH_CK(cudaStreamSynchronize(st));
            if (!c.host_ds->cond) break;
            const int save = c.launches;  // loop-body launches are counted per iteration
            launch_solve_iter(c, nf, kind, 0, 0, st);
            c.launches = save;
        }
        return TSPH_OK;
    }
    cudaStreamCaptureStatus cs;
    cudaGraph_t g;
    const cudaGraphNode_t *deps = nullptr;
    const cudaGraphEdgeData *ed = nullptr;
    size_t nd = 0;
    TSPH_CK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, &ed, &nd));
    cudaGraphConditionalHandle h;
    TSPH_CK(cudaGraphConditionalHandleCreate(&h, g, 0, 0));
    launch_solve_begin(c, kind, h, 1, st);
    TSPH_CK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, &ed, &nd));
    cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    TSPH_CK(cudaGraphAddNode(&node, g, deps, ed, nd, &np));
    TSPH_CK(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    cudaGraph_t body = np.conditional.phGraph_out[0];
    cudaStream_t bs = extra(&c)->body_stream;
    TSPH_CK(cudaStreamBeginCaptureToGraph(bs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    const int save = c.launches;
    launch_solve_iter(c, nf, kind, h, 1, bs);
    c.launches = save;
    cudaGraph_t tmp;
    TSPH_CK(cudaStreamEndCapture(bs, &tmp));
    return TSPH_OK;
}

int fbm_loop(tsph_ctx &c, int64_t nf, cudaStream_t st, bool graph) {
    if (!graph) {
        launch_fbm_begin(c, nf, 0, 0, st);
        for (;;) {
            TSPH_CK(cudaMemcpyAsync(&c.host_ds->fbm_cond, &c.ds->fbm_cond, sizeof(int), cudaMemcpyDeviceToHost, st));
            TSPH_CK(cudaStreamSynchronize(st));
            if (!c.host_ds->fbm_cond) break;
            const int save = c.launches;
            launch_fbm_pass(c, nf, 0, 0, st);
            c.launches = save;
        }
        return TSPH_OK;
    }
    cudaStreamCaptureStatus cs;
    cudaGraph_t g;
    const cudaGraphNode_t *deps = nullptr;
    const cudaGraphEdgeData *ed = nullptr;
    size_t nd = 0;
    TSPH_CK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, &ed, &nd));
    cudaGraphConditionalHandle h;
    TSPH_CK(cudaGraphConditionalHandleCreate(&h, g, 0, 0));
    launch_fbm_begin(c, nf, h, 1, st);
    TSPH_CK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, &ed, &nd));
    cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    TSPH_CK(cudaGraphAddNode(&node, g, deps, ed, nd, &np));
    TSPH_CK(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    cudaGraph_t body = np.conditional.phGraph_out[0];
    cudaStream_t bs = extra(&c)->body_stream;
    TSPH_CK(cudaStreamBeginCaptureToGraph(bs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    const int save = c.launches;
    launch_fbm_pass(c, nf, h, 1, bs);
    c.launches = save;
    cudaGraph_t tmp;
    TSPH_CK(cudaStreamEndCapture(bs, &tmp));
    return TSPH_OK;
}

// Enqueues one step (optionally preceded by cfl_condition) on `st`.
int enqueue_step(tsph_ctx &c, const tsph_set &f, const tsph_set &b, cudaStream_t st, bool with_cfl, bool graph) {
    c.launches = 0;
    launch_step_begin(c, st);
    if (with_cfl) launch_cfl(c, f, st);
    launch_grid_build(c, f, b, st);
    launch_density(c, f.n, b.n, st);
    int rc = solve(c, f.n, kSolveDiv, st, graph);
    if (rc) return rc;
    launch_advect(c, f.n, st);
    rc = solve(c, f.n, kSolveDens, st, graph);
    if (rc) return rc;
    if (c.p.fbm_enabled) {
        rc = fbm_loop(c, f.n, st, graph);
        if (rc) return rc;
    }
    launch_unsort(c, f, b, st);
    c.launches_per_step = c.launches;
    return TSPH_OK;
}

unsigned long long mix(unsigned long long h, unsigned long long v) {
    h ^= v + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
    return h;
}

void set_key(const tsph_set &f, const tsph_set &b, int with_cfl, unsigned long long out[4]) {
    unsigned long long h1 = 1469598103934665603ull, h2 = 7ull;
    const unsigned long long *pf = (const unsigned long long *)&f;
    const unsigned long long *pb = (const unsigned long long *)&b;
    for (size_t i = 0; i < sizeof(tsph_set) / 8; ++i) h1 = mix(h1, pf[i]);
    for (size_t i = 0; i < sizeof(tsph_set) / 8; ++i) h2 = mix(h2, pb[i]);
    out[0] = h1;
    out[1] = h2;
    out[2] = (unsigned long long)f.n;
    out[3] = ((unsigned long long)b.n << 1) | (unsigned long long)with_cfl;
}

int run_step(tsph_ctx *c, const tsph_set *f, const tsph_set *b, void *stream, bool with_cfl) {
    if (!c || !f || !b) return fail(TSPH_ERR_INVALID, "null argument");
    if (f->n < 0 || b->n < 0 || f->n > c->F.cap || b->n > c->B.cap)
        return fail(TSPH_ERR_CAPACITY, "part_num above the capacity given at tsph_create");
    cudaStream_t st = (cudaStream_t)stream;
    if (!c->use_graph) {
        int rc = enqueue_step(*c, *f, *b, st, with_cfl, false);
        if (rc) return rc;
        TSPH_CK(cudaGetLastError());
        c->stepped++;
        return TSPH_OK;
    }
    unsigned long long key[4];
    set_key(*f, *b, with_cfl ? 1 : 0, key);
    if (!c->exec || std::memcmp(key, c->graph_key, sizeof(key)) != 0) {
        if (c->exec) {
            cudaGraphExecDestroy(c->exec);
            c->exec = nullptr;
        }
        cudaStream_t cap = extra(c)->cap_stream;
        TSPH_CK(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
        int rc = enqueue_step(*c, *f, *b, cap, with_cfl, true);
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamEndCapture(cap, &graph);
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (e != cudaSuccess) return fail_cuda(e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&c->exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            c->exec = nullptr;
            return fail_cuda(e, "cudaGraphInstantiate");
        }
        std::memcpy(c->graph_key, key, sizeof(key));
    }
    TSPH_CK(cudaGraphLaunch(c->exec, st));
    c->stepped++;
    return TSPH_OK;
}

}  // namespace

// The extra host state lives right after the public struct in one allocation.
struct CtxBox {
    tsph_ctx c;
    CtxExtra x;
};

namespace {
CtxExtra *extra(tsph_ctx *c) { return &reinterpret_cast<CtxBox *>(c)->x; }
}  // namespace

extern "C" {

const char *tsph_version(void) { return "tichi_sph_gb300 0.1 (sm_103a)"; }

const char *tsph_last_error(void) { return g_last_error; }

}  // extern "C"

namespace tsph {
// Lets other translation units report through tsph_last_error.
void set_last_error_text(const char *msg) { std::snprintf(g_last_error, sizeof(g_last_error), "%s", msg); }
}  // namespace tsph

extern "C" {

int tsph_create(const tsph_params *p, int64_t capf, int64_t capb, tsph_ctx **out) {
    if (!p || !out) return fail(TSPH_ERR_INVALID, "null argument");
    *out = nullptr;
    if (p->dim != 2 && p->dim != 3) return fail(TSPH_ERR_INVALID, "dim must be 2 or 3");
    if (p->phase_num < 1 || p->phase_num > TSPH_MAX_PHASES) return fail(TSPH_ERR_INVALID, "phase_num out of range");
    if (p->neighb_range < 0 || p->neighb_range > 8) return fail(TSPH_ERR_INVALID, "neighb_range out of range");
    if (!(p->kernel_h > 0.f)) return fail(TSPH_ERR_INVALID, "kernel_h must be positive");
    if (p->node_num < 1 || p->node_num > 0x7ffffff0ll) return fail(TSPH_ERR_INVALID, "node_num out of range");
    if (capf < 0 || capb < 0 || capf > 0x7ffffff0ll || capb > 0x7ffffff0ll)
        return fail(TSPH_ERR_INVALID, "capacity out of range");
    if (p->cs == 0) return fail(TSPH_ERR_INVALID, "solver_cs must be nonzero");
    CtxBox *box = new (std::nothrow) CtxBox();
    if (!box) return fail(TSPH_ERR_INVALID, "out of host memory");
    tsph_ctx &c = box->c;
    Alloc &A = box->x.alloc;
    c.p = *p;
    KConst &k = c.k;
    for (int d = 0; d < 3; ++d) {
        k.lb[d] = d < p->dim ? p->lb[d] : 0.f;
        k.g[d] = d < p->dim ? p->gravity[d] : 0.f;
    }
    k.h = p->kernel_h;
    k.h2 = p->kernel_h2;
    k.inv_h = 1.f / p->kernel_h;
    k.sig = p->kernel_sig;
    k.sig_h = p->kernel_sig / p->kernel_h;
    k.node_num = p->node_num;
    k.nx = p->grid_size[0];
    k.nxny = (long long)p->grid_size[0] * (p->dim == 3 ? p->grid_size[1] : 1);
    k.R = p->neighb_range;
    k.dim = p->dim;
    k.P = p->phase_num;
    k.vfsph = p->solver_type == TSPH_VFSPH ? 1 : 0;
    k.mu = p->viscosity;
    k.gamma = p->surface_tension_gamma;
    k.fbm_c = p->fbm_convection;
    k.fbm_D = p->fbm_diffusion;
    for (int q = 0; q < kMaxP; ++q) k.rho_phase[q] = q < p->phase_num ? p->phase_rest_density[q] : 0.f;
    k.part_size = p->part_size;
    k.cfl = p->cfl_factor;
    k.cs = p->cs;
    k.iter_min = p->iter_min;
    k.iter_max = p->iter_max;
    k.fbm_max_passes = p->fbm_max_passes > 0 ? p->fbm_max_passes : 1000;
    k.div_tol = p->divergence_threshold;
    k.comp_tol = p->compression_threshold;
    k.c_coh = (float)(32.0 / 3.14159265358979323846 / ((double)p->kernel_h * p->kernel_h * p->kernel_h));

    const int64_t nn = p->node_num, P = p->phase_num;
    if (capf < 1) capf = 1;
    if (capb < 1) capb = 1;
    FluidBuf &F = c.F;
    F.cap = capf;
    F.count = A.get<int>(nn);
    F.start = A.get<int>(nn + 1);
    F.slot = A.get<int>(capf);
    F.perm = A.get<int>(capf);
    F.inv = A.get<int>(capf);
    F.pos = A.get<float4>(capf);
    F.mv = A.get<float2>(capf);
    F.mpsi = A.get<float4>(capf);
    F.rho0 = A.get<float>(capf);
    F.vel = A.get<float4>(capf);
    F.vadv = A.get<float4>(2 * capf);
    F.psiadv = A.get<float>(capf);
    F.kappa = A.get<float>(capf);
    F.acc = A.get<float4>(capf);
    F.normal = A.get<float4>(capf);
    F.W = A.get<float>(capf);
    F.rho = A.get<float>(capf);
    F.comp = A.get<float>(capf);
    F.a2 = A.get<float>(capf);
    F.a1 = A.get<float4>(capf);
    F.vf = A.get<float>(P * capf);
    F.vftmp = A.get<float>(P * capf);
    F.drift = A.get<float4>(P * capf);
    F.facc = A.get<float4>(capf);
    F.zeta = A.get<float>(capf);
    F.flagpass = A.get<int>(capf);
    k.nbr_max = p->dim == 3 ? 64 : 32;  // a multiple of 4 (blocked layout)
    F.nbr = A.get<int>((int64_t)k.nbr_max * capf);
    F.nbr_cnt = A.get<unsigned int>(capf);
    BoundBuf &B = c.B;
    B.cap = capb;
    B.count = A.get<int>(nn);
    B.start = A.get<int>(nn + 1);
    B.slot = A.get<int>(capb);
    B.perm = A.get<int>(capb);
    B.inv = A.get<int>(capb);
    B.pos = A.get<float4>(capb);
    B.mv = A.get<float2>(capb);
    B.vadv = A.get<float4>(capb);
    B.kappa = A.get<float>(capb);
    B.W = A.get<float>(capb);
    B.rho = A.get<float>(capb);
    B.comp = A.get<float>(capb);
    B.a2 = A.get<float>(capb);
    B.alpha = A.get<float>(capb);
    const int64_t nmax = capf > capb ? capf : capb;
    c.S.partials_len = 8 * (int64_t)blocks_for(nmax) + 64;  // up to 8 threads per particle
    c.S.partials = A.get<double>(c.S.partials_len);
    const int64_t nscan = (nn + 4095) / 4096 + 1;
    c.S.scan_len = 2 * nscan;
    c.S.scan_blocks = A.get<int>(c.S.scan_len);
    c.dp = A.get<DevPersist>(1);
    c.ds = A.get<DevStep>(1);
    if (A.err != cudaSuccess) {
        int rc = fail_cuda(A.err, "cudaMalloc in tsph_create");
        tsph_destroy(&c);
        return rc;
    }
    cudaError_t e = cudaMallocHost(&c.host_ds, sizeof(DevStep));
    if (e == cudaSuccess) e = cudaMallocHost(&c.host_dp, sizeof(DevPersist));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&box->x.cap_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&box->x.body_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        int rc = fail_cuda(e, "tsph_create");
        tsph_destroy(&c);
        return rc;
    }
    c.use_graph = 1;
    c.tpp = 1;
    *out = &c;
    return TSPH_OK;
}

int tsph_destroy(tsph_ctx *c) {
    if (!c) return TSPH_OK;
    CtxBox *box = reinterpret_cast<CtxBox *>(c);
    if (c->exec) cudaGraphExecDestroy(c->exec);
    for (void *p : box->x.alloc.ptrs) cudaFree(p);
    if (c->host_ds) cudaFreeHost(c->host_ds);
    if (c->host_dp) cudaFreeHost(c->host_dp);
    if (box->x.cap_stream) cudaStreamDestroy(box->x.cap_stream);
    if (box->x.body_stream) cudaStreamDestroy(box->x.body_stream);
    delete box;
    return TSPH_OK;
}

int tsph_set_graph_mode(tsph_ctx *c, int use_graph) {
    if (!c) return fail(TSPH_ERR_INVALID, "null ctx");
    c->use_graph = use_graph ? 1 : 0;
    return TSPH_OK;
}

int tsph_set_threads_per_particle(tsph_ctx *c, int tpp) {
    if (!c) return fail(TSPH_ERR_INVALID, "null ctx");
    if (tpp != 1 && tpp != 2 && tpp != 4 && tpp != 8) return fail(TSPH_ERR_INVALID, "threads per particle must be 1, 2, 4 or 8");
    if (tpp != c->tpp && c->exec) {
        cudaGraphExecDestroy(c->exec);
        c->exec = nullptr;
    }
    c->tpp = tpp;
    return TSPH_OK;
}

int tsph_cfl_condition(tsph_ctx *c, const tsph_set *f, void *stream) {
    if (!c || !f) return fail(TSPH_ERR_INVALID, "null argument");
    launch_cfl(*c, *f, (cudaStream_t)stream);
    TSPH_CK(cudaGetLastError());
    return TSPH_OK;
}

int tsph_sph_step(tsph_ctx *c, const tsph_set *f, const tsph_set *b, void *stream) {
    return run_step(c, f, b, stream, false);
}

int tsph_substep(tsph_ctx *c, const tsph_set *f, const tsph_set *b, void *stream) {
    return run_step(c, f, b, stream, true);
}

int tsph_read_stats(tsph_ctx *c, tsph_stats *out, void *stream) {
    if (!c || !out) return fail(TSPH_ERR_INVALID, "null argument");
    cudaStream_t st = (cudaStream_t)stream;
    TSPH_CK(cudaMemcpyAsync(c->host_ds, c->ds, sizeof(DevStep), cudaMemcpyDeviceToHost, st));
    TSPH_CK(cudaMemcpyAsync(c->host_dp, c->dp, sizeof(DevPersist), cudaMemcpyDeviceToHost, st));
    TSPH_CK(cudaStreamSynchronize(st));
    const DevStep &s = *c->host_ds;
    const DevPersist &d = *c->host_dp;
    std::memset(out, 0, sizeof(*out));
    out->dt = d.dt;
    out->time_count = d.time_count;
    out->compression = d.compression;
    out->kinetic_energy = s.kinetic_energy;
    out->potential_energy = s.potential_energy;
    out->div_iter = s.div_iter;
    out->incom_iter = s.incom_iter;
    out->fbm_passes = s.fbm_passes;
    out->general_flag = c->p.fbm_enabled ? s.gflag_out : 1;
    out->status = s.status;
    out->fluid_in_grid = -1;
    out->bound_in_grid = -1;
    out->steps = c->stepped;
    out->total_div_iter = d.total_div_iter;
    out->total_incom_iter = d.total_incom_iter;
    out->total_fbm_passes = d.total_fbm_passes;
    out->max_dens_compression = d.max_dens_compression;
    out->launches_per_step = c->launches_per_step;
    out->launches_per_iter = 2;
    out->launches_per_pass = 1;
    return TSPH_OK;
}

int tsph_profile_phases(tsph_ctx *c, const tsph_set *f, const tsph_set *b, int reps, float *ms_out, void *stream) {
    if (!c || !f || !b || !ms_out || reps < 1) return fail(TSPH_ERR_INVALID, "bad argument");
    if (f->n > c->F.cap || b->n > c->B.cap) return fail(TSPH_ERR_CAPACITY, "part_num above capacity");
    cudaStream_t st = (cudaStream_t)stream;
    // keep the persistent scalars (clock, counters) as they were
    TSPH_CK(cudaMemcpyAsync(c->host_dp, c->dp, sizeof(DevPersist), cudaMemcpyDeviceToHost, st));
    TSPH_CK(cudaStreamSynchronize(st));
    const DevPersist saved = *c->host_dp;
    cudaEvent_t e0, e1;
    TSPH_CK(cudaEventCreate(&e0));
    TSPH_CK(cudaEventCreate(&e1));
    const int64_t nf = f->n, nb = b->n;
    for (int ph = 0; ph < TSPH_PH_COUNT; ++ph) {
        // state every phase expects: a fresh step through the density sweep
        launch_step_begin(*c, st);
        launch_cfl(*c, *f, st);
        launch_grid_build(*c, *f, *b, st);
        launch_density(*c, nf, nb, st);
        launch_solve_begin(*c, kSolveDiv, 0, 0, st);
        if (nf > 0) launch_psi(*c, nf, st);
        TSPH_CK(cudaEventRecord(e0, st));
        for (int r = 0; r < reps; ++r) {
            switch (ph) {
                case TSPH_PH_CFL: launch_cfl(*c, *f, st); break;
                case TSPH_PH_GRID: launch_grid_build(*c, *f, *b, st); break;
                case TSPH_PH_DENSITY: launch_density(*c, nf, nb, st); break;
                case TSPH_PH_PSI: if (nf > 0) launch_psi(*c, nf, st); break;
                case TSPH_PH_VEL: if (nf > 0) launch_vel(*c, nf, kSolveDiv, 0, 0, st); break;
                case TSPH_PH_ADVECT: launch_advect(*c, nf, st); break;
                case TSPH_PH_UNSORT: launch_unsort(*c, *f, *b, st); break;
            }
        }
        TSPH_CK(cudaEventRecord(e1, st));
        TSPH_CK(cudaEventSynchronize(e1));
        float ms = 0.f;
        TSPH_CK(cudaEventElapsedTime(&ms, e0, e1));
        ms_out[ph] = ms / reps;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *c->host_dp = saved;
    TSPH_CK(cudaMemcpyAsync(c->dp, c->host_dp, sizeof(DevPersist), cudaMemcpyHostToDevice, st));
    TSPH_CK(cudaStreamSynchronize(st));
    TSPH_CK(cudaGetLastError());
    return TSPH_OK;
}

int tsph_set_state(tsph_ctx *c, double time_count, float dt, double compression, void *stream) {
    if (!c) return fail(TSPH_ERR_INVALID, "null ctx");
    k_set_state<<<1, 1, 0, (cudaStream_t)stream>>>(c->dp, time_count, dt, compression);
    TSPH_CK(cudaGetLastError());
    return TSPH_OK;
}

int tsph_neighbor_stats(tsph_ctx *c, const tsph_set *f, const tsph_set *b, int32_t *fc, uint64_t *fh, int32_t *bc,
                        uint64_t *bh, void *stream) {
    if (!c || !f || !b) return fail(TSPH_ERR_INVALID, "null argument");
    if (f->n > c->F.cap || b->n > c->B.cap) return fail(TSPH_ERR_CAPACITY, "part_num above capacity");
    cudaStream_t st = (cudaStream_t)stream;
    launch_step_begin(*c, st);
    launch_grid_build(*c, *f, *b, st);
    launch_neighbor_stats(*c, f->n, b->n, fc, fh, bc, bh, st);
    TSPH_CK(cudaGetLastError());
    TSPH_CK(cudaStreamSynchronize(st));
    return TSPH_OK;
}

}  // extern "C"
