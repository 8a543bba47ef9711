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
//
// A batch context steps many independent scenes in the same launches: every
// scene keeps its own constants, time step, solver loop state and iteration
// counts, exactly as if it ran alone, and the loops run while any scene does.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "ctx.h"
#include "tape.h"

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
    std::vector<void *> pinned;
    cudaStream_t cap_stream = nullptr;
    cudaStream_t body_stream = nullptr;
};

// The extra host state lives right after the public struct in one allocation.
struct CtxBox {
    tsph_ctx c;
    CtxExtra x;
};

CtxExtra *extra(tsph_ctx *c) { return &reinterpret_cast<CtxBox *>(c)->x; }

__global__ void k_set_state(KConst k, double time_count, float dt, double compression) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < k.n_scenes; s += gridDim.x * blockDim.x) {
        k.sp[s].time_count = time_count;
        k.sp[s].dt = dt;
        k.sp[s].compression = compression;
    }
}

// A device-side while loop: `begin` sets the condition, `body` is one iteration
// whose last block updates it.  Graph mode captures a conditional while node;
// host mode reads the condition back before every iteration.
template <class Begin, class Body>
int while_loop(tsph_ctx &c, cudaStream_t st, bool graph, const int32_t *dev_flag, int32_t *host_flag, Begin begin,
               Body body) {
    if (!graph) {
        begin(0, 0, st);
        for (;;) {
            TSPH_CK(cudaMemcpyAsync(host_flag, dev_flag, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
            TSPH_CK(cudaStreamSynchronize(st));
            if (!*host_flag) break;
            const int save = c.launches;  // loop-body launches are counted per iteration
            body(0, 0, st);
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
    begin(h, 1, st);
    TSPH_CK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, &ed, &nd));
    cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    TSPH_CK(cudaGraphAddNode(&node, g, deps, ed, nd, &np));
    TSPH_CK(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    cudaGraph_t bodyg = np.conditional.phGraph_out[0];
    cudaStream_t bs = extra(&c)->body_stream;
    TSPH_CK(cudaStreamBeginCaptureToGraph(bs, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    const int save = c.launches;
    body(h, 1, bs);
    c.launches = save;
    cudaGraph_t tmp;
    TSPH_CK(cudaStreamEndCapture(bs, &tmp));
    return TSPH_OK;
}

int solve(tsph_ctx &c, int kind, cudaStream_t st, bool graph) {
    return while_loop(
        c, st, graph, &c.k.dg->cond_any, &c.host_dg->cond_any,
        [&](cudaGraphConditionalHandle h, int u, cudaStream_t s) { launch_solve_begin(c, kind, h, u, s); },
        [&](cudaGraphConditionalHandle h, int u, cudaStream_t s) {
            if (c.rec_tape) {
                // record the iterate and kappa between the two sweeps
                launch_psi(c, s);
                launch_tape_iter(c, kind, s);
                launch_vel(c, kind, h, u, s);
            } else {
                launch_solve_iter(c, kind, h, u, s);
            }
        });
}

int fbm_loop(tsph_ctx &c, cudaStream_t st, bool graph) {
    return while_loop(
        c, st, graph, &c.k.dg->fbm_any, &c.host_dg->fbm_any,
        [&](cudaGraphConditionalHandle h, int u, cudaStream_t s) { launch_fbm_begin(c, h, u, s); },
        [&](cudaGraphConditionalHandle h, int u, cudaStream_t s) { launch_fbm_pass(c, h, u, s); });
}

// Enqueues one step (optionally preceded by cfl_condition) on `st`.
int enqueue_step(tsph_ctx &c, const tsph_set &f, const tsph_set &b, cudaStream_t st, bool with_cfl, bool graph) {
    c.launches = 0;
    launch_step_begin(c, st);
    launch_grid_build(c, f, b, st, with_cfl);
    launch_density(c, st);
    if (c.rec_tape) launch_tape_state(c, st);
    int rc = solve(c, kSolveDiv, st, graph);
    if (rc) return rc;
    launch_advect(c, st);
    if (c.rec_tape) launch_tape_vmid(c, st);
    rc = solve(c, kSolveDens, st, graph);
    if (rc) return rc;
    if (c.p.wcsph_enabled) launch_wc(c, b, st);
    if (c.p.fbm_enabled) {
        rc = fbm_loop(c, st, graph);
        if (rc) return rc;
    }
    if (c.rec_tape) launch_tape_end(c, st);
    launch_unsort(c, f, b, st);
    c.launches_per_step = c.launches;
    return TSPH_OK;
}

// Cached graphs bake the launch-time constants in: any change of those drops them.
void drop_graphs(tsph_ctx *c) {
    for (int i = 0; i < 2; ++i) {
        if (c->exec[i]) cudaGraphExecDestroy(c->exec[i]);
        c->exec[i] = nullptr;
    }
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

// Validates the caller's sets against the context and, for a single-scene
// context, makes the scene's particle counts follow them (inlets add particles).
int bind_sets(tsph_ctx *c, const tsph_set *f, const tsph_set *b) {
    if (!c || !f || !b) return fail(TSPH_ERR_INVALID, "null argument");
    if (f->n < 0 || b->n < 0) return fail(TSPH_ERR_INVALID, "negative part_num");
    SceneConst &h = c->host_sc[0];
    if (c->batch) {
        long long tf = 0, tb = 0;
        for (int s = 0; s < c->n_scenes; ++s) {
            tf += c->host_sc[s].f_n;
            tb += c->host_sc[s].b_n;
        }
        if (f->n != tf || b->n != tb)
            return fail(TSPH_ERR_CAPACITY, "particle counts differ from the scene counts given at tsph_create_batch");
        return TSPH_OK;
    }
    if (f->n > c->cap_f || b->n > c->cap_b)
        return fail(TSPH_ERR_CAPACITY, "part_num above the capacity given at tsph_create");
    if (f->n > f->capacity || b->n > b->capacity)
        return fail(TSPH_ERR_CAPACITY, "part_num above the capacity of the set's own arrays");
    if (f->n != h.f_n || b->n != h.b_n) {
        h.f_n = f->n;
        h.b_n = b->n;
        c->k.s0 = h;
        TSPH_CK(cudaMemcpy((void *)c->k.sc, c->host_sc, sizeof(SceneConst), cudaMemcpyHostToDevice));
    }
    return TSPH_OK;
}

int run_step(tsph_ctx *c, const tsph_set *f, const tsph_set *b, void *stream, bool with_cfl) {
    int rc = bind_sets(c, f, b);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if (!c->use_graph) {
        rc = enqueue_step(*c, *f, *b, st, with_cfl, false);
        if (rc) return rc;
        TSPH_CK(cudaGetLastError());
        c->stepped++;
        return TSPH_OK;
    }
    unsigned long long key[4];
    set_key(*f, *b, with_cfl ? 1 : 0, key);
    key[3] = mix(key[3], (unsigned long long)(uintptr_t)c->rec_tape);
    const int gi = c->rec_tape ? 1 : 0;
    cudaGraphExec_t &exec = c->exec[gi];
    if (!exec || std::memcmp(key, c->graph_key[gi], sizeof(key)) != 0) {
        if (exec) {
            cudaGraphExecDestroy(exec);
            exec = nullptr;
        }
        cudaStream_t cap = extra(c)->cap_stream;
        TSPH_CK(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
        rc = enqueue_step(*c, *f, *b, cap, with_cfl, true);
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamEndCapture(cap, &graph);
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (e != cudaSuccess) return fail_cuda(e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            exec = nullptr;
            return fail_cuda(e, "cudaGraphInstantiate");
        }
        std::memcpy(c->graph_key[gi], key, sizeof(key));
    }
    TSPH_CK(cudaGraphLaunch(exec, st));
    c->stepped++;
    return TSPH_OK;
}

// SceneConst of one scene from its parameters.
void make_scene(const tsph_params &p, SceneConst &c) {
    std::memset(&c, 0, sizeof(c));
    for (int d = 0; d < 3; ++d) {
        c.lb[d] = d < p.dim ? p.lb[d] : 0.f;
        c.g[d] = d < p.dim ? p.gravity[d] : 0.f;
    }
    c.h = p.kernel_h;
    c.h2 = p.kernel_h2;
    c.inv_h = 1.f / p.kernel_h;
    c.sig = p.kernel_sig;
    c.sig_h = p.kernel_sig / p.kernel_h;
    c.c_coh = (float)(32.0 / 3.14159265358979323846 / ((double)p.kernel_h * p.kernel_h * p.kernel_h));
    c.node_num = p.node_num;
    c.nx = p.grid_size[0];
    c.nxny = (long long)p.grid_size[0] * (p.dim == 3 ? p.grid_size[1] : 1);
    c.mu = p.viscosity;
    c.gamma = p.surface_tension_gamma;
    c.fbm_c = p.fbm_convection;
    c.fbm_D = p.fbm_diffusion;
    for (int q = 0; q < kMaxP; ++q) c.rho_phase[q] = q < p.phase_num ? p.phase_rest_density[q] : 0.f;
    c.part_size = p.part_size;
    c.cfl = p.cfl_factor;
    c.cs = p.cs;
    c.iter_min = p.iter_min;
    c.iter_max = p.iter_max;
    c.fbm_max_passes = p.fbm_max_passes > 0 ? p.fbm_max_passes : 1000;
    c.wc_gamma = p.wc_gamma;
    c.div_tol = p.divergence_threshold;
    c.comp_tol = p.compression_threshold;
    const long long span = 2ll * p.neighb_range;
    c.row_trim = p.grid_size[0] > span && (p.dim == 2 || p.grid_size[1] > span);
}

int check_params(const tsph_params &p) {
    if (p.dim != 2 && p.dim != 3) return fail(TSPH_ERR_INVALID, "dim must be 2 or 3");
    if (p.phase_num < 1 || p.phase_num > TSPH_MAX_PHASES) return fail(TSPH_ERR_INVALID, "phase_num out of range");
    if (p.neighb_range < 0 || p.neighb_range > 8) return fail(TSPH_ERR_INVALID, "neighb_range out of range");
    if (!(p.kernel_h > 0.f)) return fail(TSPH_ERR_INVALID, "kernel_h must be positive");
    if (p.node_num < 1 || p.node_num > 0x7ffffff0ll) return fail(TSPH_ERR_INVALID, "node_num out of range");
    if (p.cs == 0) return fail(TSPH_ERR_INVALID, "solver_cs must be nonzero");
    if (p.wcsph_enabled && p.wc_gamma == 0) return fail(TSPH_ERR_INVALID, "solver_wc_gamma must be nonzero");
    return TSPH_OK;
}

long long round_chunk(long long n) { return (n + kChunk - 1) / kChunk * kChunk; }

// Builds a context for S scenes.  batch = 0: one scene whose particle counts
// follow the caller's sets up to the capacities; batch = 1: fixed counts.
int create_impl(const tsph_params *ps, int S, const int64_t *fn, const int64_t *bn, int batch, int64_t capf,
                int64_t capb, tsph_ctx **out) {
    if (!ps || !out || S < 1) return fail(TSPH_ERR_INVALID, "null argument or no scene");
    *out = nullptr;
    for (int s = 0; s < S; ++s) {
        int rc = check_params(ps[s]);
        if (rc) return rc;
        if (ps[s].dim != ps[0].dim || ps[s].phase_num != ps[0].phase_num ||
            ps[s].solver_type != ps[0].solver_type || ps[s].neighb_range != ps[0].neighb_range ||
            ps[s].fbm_enabled != ps[0].fbm_enabled || ps[s].wcsph_enabled != ps[0].wcsph_enabled)
            return fail(TSPH_ERR_INVALID, "scenes of a batch must share dim, phase_num, solver_type, "
                                          "neighb_range, fbm_enabled and wcsph_enabled");
        if (batch && (fn[s] < 0 || bn[s] < 0)) return fail(TSPH_ERR_INVALID, "negative scene particle count");
    }
    if (!batch && (capf < 0 || capb < 0)) return fail(TSPH_ERR_INVALID, "negative capacity");
    CtxBox *box = new (std::nothrow) CtxBox();
    if (!box) return fail(TSPH_ERR_INVALID, "out of host memory");
    tsph_ctx &c = box->c;
    Alloc &A = box->x.alloc;
    c.p = ps[0];
    c.n_scenes = S;
    c.batch = batch;
    c.cap_f = capf;
    c.cap_b = capb;
    c.tpp = 1;
    c.use_graph = 1;

    std::vector<SceneConst> sc(S);
    long long cbase = 0, fslot = 0, bslot = 0, fuser = 0, buser = 0, ublk = 0;
    int st_on = 0;
    for (int s = 0; s < S; ++s) {
        make_scene(ps[s], sc[s]);
        sc[s].cbase = cbase;
        cbase += ps[s].node_num;
        const long long nf = batch ? fn[s] : 0, nb = batch ? bn[s] : 0;
        sc[s].f_user = fuser;
        sc[s].b_user = buser;
        sc[s].f_n = nf;
        sc[s].b_n = nb;
        sc[s].f_slot = fslot;
        sc[s].b_slot = bslot;
        sc[s].f_slots = round_chunk(batch ? nf : (capf > 0 ? capf : 1));
        sc[s].b_slots = round_chunk(batch ? nb : (capb > 0 ? capb : 1));
        fslot += sc[s].f_slots;
        bslot += sc[s].b_slots;
        const long long fu = batch ? nf : capf;
        sc[s].f_ublk0 = ublk;
        sc[s].f_ublks = fu > 0 ? (fu + kBlock - 1) / kBlock : 1;
        ublk += sc[s].f_ublks;
        fuser += fu;
        buser += batch ? nb : capb;
        if (ps[s].surface_tension_gamma != 0.f) st_on = 1;
    }
    if (cbase > 0x7ffffff0ll) {
        delete box;
        return fail(TSPH_ERR_INVALID, "total grid cells of the batch exceed 2^31");
    }
    c.st_on = st_on;
    // at least one chunk per set, owned by a scene without particles of that set
    const long long fcap = fslot > 0 ? fslot : kChunk, bcap = bslot > 0 ? bslot : kChunk;
    const long long nn = cbase, P = ps[0].phase_num;
    KConst &k = c.k;
    k.dim = ps[0].dim;
    k.P = ps[0].phase_num;
    k.vfsph = ps[0].solver_type == TSPH_VFSPH ? 1 : 0;
    k.R = ps[0].neighb_range;
    k.nbr_max = ps[0].dim == 3 ? 64 : 32;  // a multiple of 4 (blocked layout)
    k.n_scenes = S;
    k.total_nodes = nn;
    k.f_slots = fcap;
    k.b_slots = bcap;

    std::vector<int> fchunk(fcap / kChunk, 0), bchunk(bcap / kChunk, 0);
    std::vector<int> fus(fuser > 0 ? fuser : 1, 0), bus(buser > 0 ? buser : 1, 0);
    std::vector<int> fub(ublk, 0);
    for (int s = 0; s < S; ++s) {
        for (long long i = 0; i < sc[s].f_ublks; ++i) fub[sc[s].f_ublk0 + i] = s;
        for (long long i = sc[s].f_slot / kChunk; i < (sc[s].f_slot + sc[s].f_slots) / kChunk; ++i) fchunk[i] = s;
        for (long long i = sc[s].b_slot / kChunk; i < (sc[s].b_slot + sc[s].b_slots) / kChunk; ++i) bchunk[i] = s;
        const long long fu = batch ? sc[s].f_n : capf, bu = batch ? sc[s].b_n : capb;
        for (long long i = 0; i < fu; ++i) fus[sc[s].f_user + i] = s;
        for (long long i = 0; i < bu; ++i) bus[sc[s].b_user + i] = s;
    }
    if (fslot == 0)  // all scenes are without fluid: the chunk belongs to one of them
        for (auto &v : fchunk) v = 0;

    FluidBuf &F = c.F;
    F.cap = fcap;
    F.count = A.get<int>(nn);
    F.start = A.get<int>(nn + 1);
    F.slot = A.get<int>((long long)fus.size());
    F.inv = A.get<int>((long long)fus.size());
    F.perm = A.get<int>(fcap);
    F.perm_u = A.get<int>(fcap);
    F.pos = A.get<float4>(fcap);
    F.mv = A.get<float2>(fcap);
    F.mpsi = A.get<float4>(fcap);
    F.psilo = A.get<float>(fcap);
    F.rho0 = A.get<float>(fcap);
    F.vel = A.get<float4>(fcap);
    F.vadv = A.get<float4>(2 * fcap);
    F.psiadv = A.get<float>(fcap);
    F.kappa = A.get<float>(fcap);
    F.acc = A.get<float4>(fcap);
    F.normal = A.get<float4>(fcap);
    F.dens = A.get<float4>(fcap);
    F.a1 = A.get<float4>(fcap);
    F.vf = A.get<float>(P * fcap);
    F.vftmp = A.get<float>(P * fcap);
    F.drift = A.get<float4>(P * fcap);
    F.facc = A.get<float4>(fcap);
    F.zeta = A.get<float>(fcap);
    F.flagpass = A.get<int>(fcap);
    F.nbr = A.get<int>((long long)k.nbr_max * fcap);
    F.pk = A.get<float4>(fcap);
    F.nbr_cnt = A.get<unsigned int>(fcap);
    F.wcp = ps[0].wcsph_enabled ? A.get<float2>(fcap) : nullptr;
    BoundBuf &B = c.B;
    B.cap = bcap;
    B.count = A.get<int>(nn);
    B.start = A.get<int>(nn + 1);
    B.slot = A.get<int>((long long)bus.size());
    B.inv = A.get<int>((long long)bus.size());
    B.perm = A.get<int>(bcap);
    B.perm_u = A.get<int>(bcap);
    B.pos = A.get<float4>(bcap);
    B.mv = A.get<float2>(bcap);
    B.vadv = A.get<float4>(bcap);
    B.kappa = A.get<float>(bcap);
    B.dens = A.get<float4>(bcap);
    B.alpha = A.get<float>(bcap);
    B.pk = A.get<float4>(bcap);
    B.bb = A.get<float4>(bcap);
    B.wcp2 = ps[0].wcsph_enabled ? A.get<float>(bcap) : nullptr;
    c.S.partials_len = 2 * 8 * ((fcap + bcap) / kBlock) + 2 * ublk + 64;  // up to 8 threads per particle
    c.S.partials = A.get<double>(c.S.partials_len);
    const int64_t nscan = (nn + 4095) / 4096 + 1;
    c.S.scan_len = 2 * nscan;
    c.S.scan_blocks = A.get<int>(c.S.scan_len);
    SceneConst *d_sc = A.get<SceneConst>(S);
    k.sp = A.get<ScenePersist>(S);
    k.ss = A.get<SceneStep>(S);
    k.dg = A.get<DevGlobal>(1);
    int *d_fchunk = A.get<int>((long long)fchunk.size());
    int *d_bchunk = A.get<int>((long long)bchunk.size());
    int *d_fus = A.get<int>((long long)fus.size());
    int *d_bus = A.get<int>((long long)bus.size());
    int *d_fub = A.get<int>(ublk);
    k.sc = d_sc;
    k.f_chunk_scene = d_fchunk;
    k.b_chunk_scene = d_bchunk;
    k.f_user_scene = d_fus;
    k.b_user_scene = d_bus;
    k.f_ublock_scene = d_fub;
    k.f_ublocks = ublk;
    k.s0 = sc[0];
    cudaError_t e = A.err;
    if (e == cudaSuccess) e = cudaMemcpy(d_sc, sc.data(), sizeof(SceneConst) * S, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_fchunk, fchunk.data(), sizeof(int) * fchunk.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_bchunk, bchunk.data(), sizeof(int) * bchunk.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_fus, fus.data(), sizeof(int) * fus.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_bus, bus.data(), sizeof(int) * bus.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_fub, fub.data(), sizeof(int) * ublk, cudaMemcpyHostToDevice);
    void *hp = nullptr;
    if (e == cudaSuccess) e = cudaMallocHost(&hp, sizeof(SceneConst) * S);
    if (e == cudaSuccess) {
        box->x.pinned.push_back(hp);
        c.host_sc = (SceneConst *)hp;
        std::memcpy(c.host_sc, sc.data(), sizeof(SceneConst) * S);
        e = cudaMallocHost(&hp, sizeof(SceneStep) * S);
    }
    if (e == cudaSuccess) {
        box->x.pinned.push_back(hp);
        c.host_ss = (SceneStep *)hp;
        e = cudaMallocHost(&hp, sizeof(ScenePersist) * S);
    }
    if (e == cudaSuccess) {
        box->x.pinned.push_back(hp);
        c.host_sp = (ScenePersist *)hp;
        e = cudaMallocHost(&hp, sizeof(DevGlobal));
    }
    if (e == cudaSuccess) {
        box->x.pinned.push_back(hp);
        c.host_dg = (DevGlobal *)hp;
        e = cudaStreamCreateWithFlags(&box->x.cap_stream, cudaStreamNonBlocking);
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&box->x.body_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c.side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c.ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c.ev_join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        int rc = fail_cuda(e, "tsph_create");
        tsph_destroy(&c);
        return rc;
    }
    *out = &c;
    return TSPH_OK;
}

void fill_stats(const tsph_ctx *c, int s, tsph_stats *out) {
    const SceneStep &st = c->host_ss[s];
    const ScenePersist &d = c->host_sp[s];
    std::memset(out, 0, sizeof(*out));
    out->dt = d.dt;
    out->time_count = d.time_count;
    out->compression = d.compression;
    out->kinetic_energy = st.kinetic_energy;
    out->potential_energy = st.potential_energy;
    out->div_iter = st.div_iter;
    out->incom_iter = st.incom_iter;
    out->fbm_passes = st.fbm_passes;
    out->general_flag = c->p.fbm_enabled ? st.gflag_out : 1;
    out->status = st.status;
    out->fluid_in_grid = st.f_in;
    out->bound_in_grid = st.b_in;
    out->steps = d.steps;
    out->total_div_iter = d.total_div_iter;
    out->total_incom_iter = d.total_incom_iter;
    out->total_fbm_passes = d.total_fbm_passes;
    out->max_dens_compression = d.max_dens_compression;
    out->launches_per_step = c->launches_per_step;
    out->launches_per_iter = 2;
    out->launches_per_pass = 1;
}

}  // namespace

namespace tsph {
// Lets other translation units report through tsph_last_error.
void set_last_error_text(const char *msg) { std::snprintf(g_last_error, sizeof(g_last_error), "%s", msg); }
}  // namespace tsph

extern "C" {

const char *tsph_version(void) { return "tichi_sph_gb300 0.2 (sm_103a)"; }

const char *tsph_last_error(void) { return g_last_error; }

int tsph_create(const tsph_params *p, int64_t capf, int64_t capb, tsph_ctx **out) {
    if (capf > 0x7fff0000ll || capb > 0x7fff0000ll) return fail(TSPH_ERR_INVALID, "capacity out of range");
    return create_impl(p, 1, nullptr, nullptr, 0, capf, capb, out);
}

int tsph_create_batch(const tsph_params *scenes, int n_scenes, const int64_t *fluid_counts,
                      const int64_t *bound_counts, tsph_ctx **out) {
    if (!scenes || !fluid_counts || !bound_counts || n_scenes < 1)
        return fail(TSPH_ERR_INVALID, "null argument or no scene");
    long long tf = 0, tb = 0;
    for (int s = 0; s < n_scenes; ++s) {
        tf += fluid_counts[s];
        tb += bound_counts[s];
    }
    if (tf > 0x7fff0000ll || tb > 0x7fff0000ll) return fail(TSPH_ERR_INVALID, "batch particle count out of range");
    return create_impl(scenes, n_scenes, fluid_counts, bound_counts, 1, 0, 0, out);
}

int tsph_destroy(tsph_ctx *c) {
    if (!c) return TSPH_OK;
    CtxBox *box = reinterpret_cast<CtxBox *>(c);
    drop_graphs(c);
    for (void *p : box->x.alloc.ptrs) cudaFree(p);
    for (void *p : box->x.pinned) cudaFreeHost(p);
    if (box->x.cap_stream) cudaStreamDestroy(box->x.cap_stream);
    if (box->x.body_stream) cudaStreamDestroy(box->x.body_stream);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
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
    if (tpp != 1 && tpp != 2 && tpp != 4 && tpp != 8)
        return fail(TSPH_ERR_INVALID, "threads per particle must be 1, 2, 4 or 8");
    if (tpp != c->tpp) drop_graphs(c);
    c->tpp = tpp;
    return TSPH_OK;
}

int tsph_cfl_condition(tsph_ctx *c, const tsph_set *f, void *stream) {
    if (!c || !f) return fail(TSPH_ERR_INVALID, "null argument");
    cudaStream_t st = (cudaStream_t)stream;
    TSPH_CK(cudaMemsetAsync(c->k.dg->ticket, 0, sizeof(unsigned int), st));
    launch_cfl(*c, *f, st);
    TSPH_CK(cudaGetLastError());
    return TSPH_OK;
}

int tsph_sph_step(tsph_ctx *c, const tsph_set *f, const tsph_set *b, void *stream) {
    return run_step(c, f, b, stream, false);
}

int tsph_substep(tsph_ctx *c, const tsph_set *f, const tsph_set *b, void *stream) {
    return run_step(c, f, b, stream, true);
}

// ----------------------------------------------------------- kernel-level composition
// The phases of enqueue_step one call at a time; the caller runs the solver and
// volume-fraction loops on the host, as main.py:199-250 does.

static int kl_check(tsph_ctx *c, const char *what) {
    if (!c) return fail(TSPH_ERR_INVALID, "null ctx");
    if (c->n_scenes != 1) {
        std::snprintf(g_last_error, sizeof(g_last_error), "%s: kernel-level calls take a one-scene context", what);
        return TSPH_ERR_INVALID;
    }
    return TSPH_OK;
}

static int kl_state(const char *what, const char *need) {
    std::snprintf(g_last_error, sizeof(g_last_error), "%s called out of order: %s", what, need);
    return TSPH_ERR_STATE;
}

// scene 0's per-step scalars, after the work enqueued on `st`
static int kl_read_step(tsph_ctx *c, cudaStream_t st) {
    TSPH_CK(cudaMemcpyAsync(c->host_ss, c->k.ss, sizeof(SceneStep), cudaMemcpyDeviceToHost, st));
    TSPH_CK(cudaMemcpyAsync(c->host_sp, c->k.sp, sizeof(ScenePersist), cudaMemcpyDeviceToHost, st));
    TSPH_CK(cudaStreamSynchronize(st));
    return TSPH_OK;
}

int tsph_grid_build(tsph_ctx *c, const tsph_set *f, const tsph_set *b, void *stream) {
    int rc = kl_check(c, "tsph_grid_build");
    if (rc) return rc;
    rc = bind_sets(c, f, b);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    launch_step_begin(*c, st);
    launch_grid_build(*c, *f, *b, st, false);
    TSPH_CK(cudaGetLastError());
    c->kl_phase = 1;
    c->kl_psi = 0;
    c->kl_fbm = 0;
    return TSPH_OK;
}

int tsph_density_alpha(tsph_ctx *c, void *stream) {
    int rc = kl_check(c, "tsph_density_alpha");
    if (rc) return rc;
    if (c->kl_phase != 1) return kl_state("tsph_density_alpha", "it follows tsph_grid_build");
    cudaStream_t st = (cudaStream_t)stream;
    launch_density(*c, st);
    launch_solve_begin(*c, kSolveDiv, 0, 0, st);
    TSPH_CK(cudaGetLastError());
    c->kl_phase = 2;
    return TSPH_OK;
}

static int kl_solve_phase(tsph_ctx *c, int kind, const char *what) {
    if (kind != TSPH_SOLVE_DIV && kind != TSPH_SOLVE_DENS) return fail(TSPH_ERR_INVALID, "unknown solve kind");
    if (kind == TSPH_SOLVE_DIV && c->kl_phase != 2)
        return kl_state(what, "the divergence solve runs between tsph_density_alpha and tsph_nonpressure");
    if (kind == TSPH_SOLVE_DENS && c->kl_phase != 3)
        return kl_state(what, "the density solve runs between tsph_nonpressure and the weakly compressible, "
                              "volume-fraction or update calls");
    return TSPH_OK;
}

int tsph_adv_psi(tsph_ctx *c, int kind, double *compression_out, void *stream) {
    int rc = kl_check(c, "tsph_adv_psi");
    if (rc) return rc;
    rc = kl_solve_phase(c, kind, "tsph_adv_psi");
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    launch_psi(*c, st, 1);
    TSPH_CK(cudaGetLastError());
    c->kl_psi = 1;
    if (compression_out) {
        rc = kl_read_step(c, st);
        if (rc) return rc;
        *compression_out = c->host_ss[0].psi_sum / (double)c->host_sc[0].f_n;
    }
    return TSPH_OK;
}

int tsph_update_vel_adv(tsph_ctx *c, int kind, void *stream) {
    int rc = kl_check(c, "tsph_update_vel_adv");
    if (rc) return rc;
    rc = kl_solve_phase(c, kind, "tsph_update_vel_adv");
    if (rc) return rc;
    if (!c->kl_psi) return kl_state("tsph_update_vel_adv", "each sweep B follows a sweep A (tsph_adv_psi)");
    launch_vel(*c, kind == TSPH_SOLVE_DIV ? kSolveDiv : kSolveDens, 0, 0, (cudaStream_t)stream, 1);
    TSPH_CK(cudaGetLastError());
    c->kl_psi = 0;
    return TSPH_OK;
}

int tsph_solve(tsph_ctx *c, int kind, double tol, int32_t it_min, int32_t it_max, int32_t *it_out, double *err_out,
               void *stream) {
    int rc = kl_check(c, "tsph_solve");
    if (rc) return rc;
    rc = kl_solve_phase(c, kind, "tsph_solve");
    if (rc) return rc;
    const SceneConst &h = c->host_sc[0];
    if (tol < 0.0) tol = kind == TSPH_SOLVE_DIV ? (double)h.div_tol : (double)h.comp_tol;
    if (it_min < 0) it_min = h.iter_min;
    if (it_max < 0) it_max = h.iter_max;
    cudaStream_t st = (cudaStream_t)stream;
    // the compression the first loop test reads: the last solve's (main.py:201, 222)
    rc = kl_read_step(c, st);
    if (rc) return rc;
    double comp = c->host_sp[0].compression;
    int it = 0;
    const int dk = kind == TSPH_SOLVE_DIV ? kSolveDiv : kSolveDens;
    while (it < it_min || comp > tol) {
        launch_psi(*c, st, 1);
        launch_vel(*c, dk, 0, 0, st, 1);
        TSPH_CK(cudaGetLastError());
        rc = kl_read_step(c, st);
        if (rc) return rc;
        comp = c->host_sp[0].compression;
        ++it;
        if (it > it_max) {
            launch_status_or(*c, kind == TSPH_SOLVE_DIV ? TSPH_ST_DIV_ITER_CAP : TSPH_ST_DENS_ITER_CAP, st);
            break;
        }
    }
    c->kl_psi = 0;
    if (it_out) *it_out = it;
    if (err_out) *err_out = comp;
    TSPH_CK(cudaGetLastError());
    return TSPH_OK;
}

int tsph_nonpressure(tsph_ctx *c, int32_t terms, void *stream) {
    int rc = kl_check(c, "tsph_nonpressure");
    if (rc) return rc;
    if (c->kl_phase != 2) return kl_state("tsph_nonpressure", "it follows tsph_density_alpha and the divergence solve");
    if (terms & ~TSPH_TERM_ALL) return fail(TSPH_ERR_INVALID, "tsph_nonpressure: unknown TSPH_TERM_* bits");
    cudaStream_t st = (cudaStream_t)stream;
    launch_advect(*c, st, terms);
    launch_solve_begin(*c, kSolveDens, 0, 0, st);  // the predicted v_adv starts the density solve
    TSPH_CK(cudaGetLastError());
    c->kl_phase = 3;
    c->kl_psi = 0;
    return TSPH_OK;
}

int tsph_wc_pressure(tsph_ctx *c, const tsph_set *b, void *stream) {
    int rc = kl_check(c, "tsph_wc_pressure");
    if (rc) return rc;
    if (!b) return fail(TSPH_ERR_INVALID, "null argument");
    if (!c->p.wcsph_enabled) return fail(TSPH_ERR_INVALID, "tsph_wc_pressure: the context has wcsph_enabled = 0");
    if (c->kl_phase != 3) return kl_state("tsph_wc_pressure", "it follows the density solve");
    launch_wc(*c, *b, (cudaStream_t)stream);
    TSPH_CK(cudaGetLastError());
    c->kl_phase = 4;
    return TSPH_OK;
}

int tsph_fbm_pass(tsph_ctx *c, int32_t *general_flag_out, void *stream) {
    int rc = kl_check(c, "tsph_fbm_pass");
    if (rc) return rc;
    if (!c->p.fbm_enabled) return fail(TSPH_ERR_INVALID, "tsph_fbm_pass: the context has fbm_enabled = 0");
    if (c->kl_phase < 3 || c->kl_phase > 5)
        return kl_state("tsph_fbm_pass", "the volume-fraction loop follows the density solve");
    cudaStream_t st = (cudaStream_t)stream;
    if (!c->kl_fbm) {
        launch_fbm_begin(*c, 0, 0, st);
        c->kl_fbm = 1;
    }
    launch_fbm_pass(*c, 0, 0, st);
    TSPH_CK(cudaGetLastError());
    c->kl_phase = 5;
    rc = kl_read_step(c, st);
    if (rc) return rc;
    if (general_flag_out) *general_flag_out = c->host_ss[0].gflag_out;
    return TSPH_OK;
}

int tsph_update(tsph_ctx *c, const tsph_set *f, const tsph_set *b, void *stream) {
    int rc = kl_check(c, "tsph_update");
    if (rc) return rc;
    if (c->kl_phase < 2) return kl_state("tsph_update", "it ends a step begun by tsph_grid_build and tsph_density_alpha");
    rc = bind_sets(c, f, b);
    if (rc) return rc;
    launch_unsort(*c, *f, *b, (cudaStream_t)stream);
    TSPH_CK(cudaGetLastError());
    c->kl_phase = 0;
    c->stepped++;
    return TSPH_OK;
}

int tsph_read_scene_stats(tsph_ctx *c, int first, int count, tsph_stats *out, void *stream) {
    if (!c || !out || first < 0 || count < 0 || first + count > c->n_scenes)
        return fail(TSPH_ERR_INVALID, "bad scene range");
    cudaStream_t st = (cudaStream_t)stream;
    TSPH_CK(cudaMemcpyAsync(c->host_ss, c->k.ss, sizeof(SceneStep) * c->n_scenes, cudaMemcpyDeviceToHost, st));
    TSPH_CK(cudaMemcpyAsync(c->host_sp, c->k.sp, sizeof(ScenePersist) * c->n_scenes, cudaMemcpyDeviceToHost, st));
    TSPH_CK(cudaStreamSynchronize(st));
    for (int i = 0; i < count; ++i) fill_stats(c, first + i, out + i);
    return TSPH_OK;
}

int tsph_read_stats(tsph_ctx *c, tsph_stats *out, void *stream) {
    return tsph_read_scene_stats(c, 0, 1, out, stream);
}

int tsph_profile_phases(tsph_ctx *c, const tsph_set *f, const tsph_set *b, int reps, float *ms_out, void *stream) {
    if (!ms_out || reps < 1) return fail(TSPH_ERR_INVALID, "bad argument");
    int rc = bind_sets(c, f, b);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const int S = c->n_scenes;
    // keep the persistent scalars (clock, counters) as they were
    std::vector<ScenePersist> saved(S);
    TSPH_CK(cudaMemcpyAsync(saved.data(), c->k.sp, sizeof(ScenePersist) * S, cudaMemcpyDeviceToHost, st));
    TSPH_CK(cudaStreamSynchronize(st));
    cudaEvent_t e0, e1;
    TSPH_CK(cudaEventCreate(&e0));
    TSPH_CK(cudaEventCreate(&e1));
    for (int ph = 0; ph < TSPH_PH_COUNT; ++ph) {
        // state every phase expects: a fresh step through the first Jacobi sweep
        launch_step_begin(*c, st);
        launch_cfl(*c, *f, st);
        launch_grid_build(*c, *f, *b, st);
        launch_density(*c, st);
        launch_solve_begin(*c, kSolveDiv, 0, 0, st);
        launch_psi(*c, st);
        // the density sweep did the first psi iteration's work: time full sweeps
        if (ph == TSPH_PH_PSI) launch_clear_psi_ready(*c, st);
        TSPH_CK(cudaEventRecord(e0, st));
        for (int r = 0; r < reps; ++r) {
            switch (ph) {
                case TSPH_PH_CFL: launch_cfl(*c, *f, st); break;
                case TSPH_PH_GRID: launch_grid_build(*c, *f, *b, st); break;
                case TSPH_PH_DENSITY: launch_density(*c, st); break;
                case TSPH_PH_PSI: launch_psi(*c, st); break;
                case TSPH_PH_VEL:
                    launch_solve_begin(*c, kSolveDiv, 0, 0, st);  // keep every scene running
                    launch_vel(*c, kSolveDiv, 0, 0, st);
                    break;
                case TSPH_PH_ADVECT: launch_advect(*c, st); break;
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
    TSPH_CK(cudaMemcpyAsync(c->k.sp, saved.data(), sizeof(ScenePersist) * S, cudaMemcpyHostToDevice, st));
    TSPH_CK(cudaStreamSynchronize(st));
    TSPH_CK(cudaGetLastError());
    return TSPH_OK;
}

int tsph_set_state(tsph_ctx *c, double time_count, float dt, double compression, void *stream) {
    if (!c) return fail(TSPH_ERR_INVALID, "null ctx");
    k_set_state<<<(c->n_scenes + 127) / 128, 128, 0, (cudaStream_t)stream>>>(c->k, time_count, dt, compression);
    TSPH_CK(cudaGetLastError());
    return TSPH_OK;
}

int tsph_substep_record(tsph_ctx *c, const tsph_set *f, const tsph_set *b, tsph_tape *t, int slot, void *stream) {
    if (!c || !t || t->ctx != c) return fail(TSPH_ERR_INVALID, "tape does not belong to this context");
    if (slot < 0 || slot >= t->a.slots) return fail(TSPH_ERR_INVALID, "tape slot out of range");
    int rc = tape_begin(*t, slot, (cudaStream_t)stream);
    if (rc) return rc;
    c->rec_tape = t;
    rc = run_step(c, f, b, stream, true);
    c->rec_tape = nullptr;
    return rc;
}

int tsph_density_record(tsph_ctx *c, const tsph_set *f, const tsph_set *b, tsph_tape *t, int slot, float *out,
                        void *stream) {
    if (!c || !t || t->ctx != c) return fail(TSPH_ERR_INVALID, "tape does not belong to this context");
    if (slot < 0 || slot >= t->a.slots) return fail(TSPH_ERR_INVALID, "tape slot out of range");
    if (!out) return fail(TSPH_ERR_INVALID, "null output");
    int rc = bind_sets(c, f, b);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    rc = tape_begin(*t, slot, st);
    if (rc) return rc;
    c->rec_tape = t;
    launch_step_begin(*c, st);
    launch_grid_build(*c, *f, *b, st);
    launch_density(*c, st);
    launch_tape_state(*c, st);
    c->rec_tape = nullptr;
    launch_density_out(*c, out, st);
    TSPH_CK(cudaGetLastError());
    return TSPH_OK;
}

int tsph_set_viscosity(tsph_ctx *c, int scene, float viscosity) {
    if (!c) return fail(TSPH_ERR_INVALID, "null ctx");
    if (scene < 0 || scene >= c->n_scenes) return fail(TSPH_ERR_INVALID, "scene out of range");
    SceneConst &h = c->host_sc[scene];
    if (h.mu == viscosity) return TSPH_OK;
    h.mu = viscosity;
    if (scene == 0) c->k.s0.mu = viscosity;
    TSPH_CK(cudaMemcpy((void *)(c->k.sc + scene), &h, sizeof(SceneConst), cudaMemcpyHostToDevice));
    drop_graphs(c);  // the one-scene kernels read mu from the launch's constant bank
    return TSPH_OK;
}

int tsph_neighbor_stats(tsph_ctx *c, const tsph_set *f, const tsph_set *b, int32_t *fc, uint64_t *fh, int32_t *bc,
                        uint64_t *bh, void *stream) {
    int rc = bind_sets(c, f, b);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    launch_step_begin(*c, st);
    launch_grid_build(*c, *f, *b, st);
    launch_neighbor_stats(*c, fc, fh, bc, bh, 0, st);
    TSPH_CK(cudaGetLastError());
    TSPH_CK(cudaStreamSynchronize(st));
    return TSPH_OK;
}

int tsph_candidate_stats(tsph_ctx *c, const tsph_set *f, const tsph_set *b, int32_t *fc, int32_t *bc,
                         void *stream) {
    if (!fc || !bc) return fail(TSPH_ERR_INVALID, "null output");
    int rc = bind_sets(c, f, b);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    launch_step_begin(*c, st);
    launch_grid_build(*c, *f, *b, st);
    launch_neighbor_stats(*c, fc, nullptr, bc, nullptr, 1, st);
    TSPH_CK(cudaGetLastError());
    TSPH_CK(cudaStreamSynchronize(st));
    return TSPH_OK;
}

}  // extern "C"
