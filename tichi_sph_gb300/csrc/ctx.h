// Solver context and the host-side launchers of each kernel group.
#pragma once

#include <cuda_runtime.h>

#include <utility>

#include "common.cuh"

struct tsph_ctx {
    tsph_params p;            // parameters of scene 0 (features shared by every scene)
    tsph::KConst k;
    tsph::FluidBuf F;
    tsph::BoundBuf B;
    tsph::Scratch S;
    tsph::SceneConst *host_sc;  // host copy of the scene table (pinned)
    tsph::SceneStep *host_ss;   // pinned mirrors for host-loop mode and stats
    tsph::ScenePersist *host_sp;
    tsph::DevGlobal *host_dg;
    int n_scenes;
    int batch;                // 0: one scene whose particle counts follow the caller's sets
    int st_on;                // some scene has surface tension
    int use_graph;
    int stepped;
    // cached per-substep graphs (plain, recording), keyed on the particle counts,
    // array pointers and the recording tape
    cudaGraphExec_t exec[2];
    unsigned long long graph_key[2][4];
    tsph_tape *rec_tape;      // non-null while a recorded step is enqueued
    int launches;             // kernel launches enqueued (counted by the launchers)
    int launches_per_step;    // top-level kernels of the last enqueued step
    int tpp;                  // threads per particle of the list sweeps (1, 2, 4, 8)
    // second stream for the boundary set's share of a phase (fork_side / join_side)
    cudaStream_t side;
    cudaEvent_t ev_fork, ev_join;
    // kernel-level composition (tsph_grid_build ... tsph_update): how far the
    // step has got (0: none in progress, 1 grid built, 2 density done, 3
    // non-pressure forces done, 4 weakly compressible block done, 5 in the
    // volume-fraction loop), whether a sweep A awaits its sweep B, and whether
    // the volume-fraction loop has begun
    int kl_phase, kl_psi, kl_fbm;
    // particle capacities given at create (the caller-order tables are this long)
    int64_t cap_f, cap_b;
};

namespace tsph {

// A kernel launch with programmatic stream serialisation: the kernel may be
// scheduled before the one ahead of it in the stream has drained, and waits
// for it in pdl_entry() (common.cuh), its first statement -- every kernel
// launched this way has it.  Only outside a stream capture (host-driven loops,
// the kernel-level entries): measured at 1M particles, stream launches gained
// (grid 124 -> 114 us, velocity sweep 80 -> 75 us per launch) while the same
// edges in the substep's CUDA graph made it slower (1.469 -> 1.487 ms), so
// graphs get plain launches.
template <typename... KArgs, typename... Args>
inline void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t st, Args &&...args) {
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(st, &cap);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = cap == cudaStreamCaptureStatusNone ? 1 : 0;
    cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}
#define TSPH_LAUNCH(K, G, B, S, ...) ::tsph::launch_pdl(K, dim3(G), dim3(B), S, __VA_ARGS__)

enum SolveKind { kSolveDiv = 0, kSolveDens = 1 };

// grid.cu
// fork_side: the side stream waits for `st`; join_side: `st` waits for the side
// stream.  Inside a stream capture the pair becomes two branches of the graph.
void fork_side(tsph_ctx &c, cudaStream_t st);
void join_side(tsph_ctx &c, cudaStream_t st);
void launch_step_begin(tsph_ctx &c, cudaStream_t st);
void launch_cfl(tsph_ctx &c, const tsph_set &f, cudaStream_t st);
// with_cfl: cfl_condition runs first on the side stream, beside the fluid's encode
void launch_grid_build(tsph_ctx &c, const tsph_set &f, const tsph_set &b, cudaStream_t st, bool with_cfl = false);
void launch_unsort(tsph_ctx &c, const tsph_set &f, const tsph_set &b, cudaStream_t st);
void launch_neighbor_stats(tsph_ctx &c, int32_t *fc, uint64_t *fh, int32_t *bc, uint64_t *bh, int cand,
                           cudaStream_t st);

// sweeps.cu
void launch_density(tsph_ctx &c, cudaStream_t st);
void launch_clear_psi_ready(tsph_ctx &c, cudaStream_t st);
void launch_solve_begin(tsph_ctx &c, int kind, cudaGraphConditionalHandle h, int use_cond, cudaStream_t st);
void launch_solve_iter(tsph_ctx &c, int kind, cudaGraphConditionalHandle h, int use_cond, cudaStream_t st);
// force = 1: the host runs the solver loop (kernel-level calls); see k_psi / k_vel
void launch_psi(tsph_ctx &c, cudaStream_t st, int force = 0);
void launch_vel(tsph_ctx &c, int kind, cudaGraphConditionalHandle h, int use_cond, cudaStream_t st, int force = 0);
// terms: TSPH_TERM_* bits of the non-pressure forces to apply
void launch_advect(tsph_ctx &c, cudaStream_t st, int terms = TSPH_TERM_ALL);
// ORs status bits into scene 0's step status (host-driven loops that hit their cap)
void launch_status_or(tsph_ctx &c, int bits, cudaStream_t st);

// wcsph.cu
void launch_wc(tsph_ctx &c, const tsph_set &b, cudaStream_t st);

// adjoint.cu: recording hooks of the forward step
void launch_tape_state(tsph_ctx &c, cudaStream_t st);
void launch_tape_iter(tsph_ctx &c, int kind, cudaStream_t st);
void launch_tape_vmid(tsph_ctx &c, cudaStream_t st);
void launch_tape_end(tsph_ctx &c, cudaStream_t st);
int tape_begin(tsph_tape &t, int slot, cudaStream_t st);
void launch_density_out(tsph_ctx &c, float *out, cudaStream_t st);

// fbm.cu
void launch_fbm_begin(tsph_ctx &c, cudaGraphConditionalHandle h, int use_cond, cudaStream_t st);
void launch_fbm_pass(tsph_ctx &c, cudaGraphConditionalHandle h, int use_cond, cudaStream_t st);

}  // namespace tsph
