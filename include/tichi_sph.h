/*
 * tichi_sph.h -- C ABI of the GB300 (sm_103a) SPH hot path.
 *
 * Drop-in boundary for the per-substep solver of Tichi_SPH.  Every entry point
 * takes plain C types: device pointers to particle arrays that the caller owns
 * (the host side keeps them as PyTorch CUDA tensors), sizes, and a CUDA stream
 * passed as `void *` (a `cudaStream_t`; NULL = legacy default stream).  No entry
 * point allocates memory except tsph_create.  All calls are stream-ordered; only
 * tsph_read_stats and tsph_neighbor_stats synchronise the stream.
 *
 * Each declaration names the reference interface it replaces (paths are within
 * the Tichi_SPH project).
 */
#ifndef TICHI_SPH_H
#define TICHI_SPH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TSPH_MAX_PHASES 8

/* Return codes.  The reference raises Python exceptions only for configuration
 * and scenario errors (sph_config.py:13-24, main.py:56,73-74); the host wrapper
 * maps these codes onto RuntimeError. */
enum {
    TSPH_OK = 0,
    TSPH_ERR_INVALID = 1,   /* bad argument or parameter */
    TSPH_ERR_CAPACITY = 2,  /* part_num above the capacity given at create */
    TSPH_ERR_CUDA = 3,      /* a CUDA runtime call failed */
    TSPH_ERR_STATE = 4      /* call order violated (e.g. stats before a step) */
};

/* Bits of tsph_stats.status (informational; a step still completes). */
enum {
    TSPH_ST_NONFINITE_POS = 1,   /* a position was NaN/inf or its cell overflowed */
    TSPH_ST_DIV_ITER_CAP = 2,    /* divergence solve stopped at iter_max (main.py:212-213) */
    TSPH_ST_DENS_ITER_CAP = 4,   /* density solve stopped at iter_max (main.py:233-234) */
    TSPH_ST_FBM_PASS_CAP = 8,    /* volume-fraction pass loop stopped at fbm_max_passes */
    TSPH_ST_OUTSIDE_GRID = 16    /* some particle had no valid cell (sph_obj.py:305,319) */
};

enum { TSPH_DFSPH = 0, TSPH_VFSPH = 1 };

/* Solver constants.  Replaces the `Config` singleton, sph_config.py:83-235.
 * Values are the f32 values the reference's Taichi fields hold. */
typedef struct tsph_params {
    int32_t dim;            /* 2 or 3 (sim_dim) */
    int32_t phase_num;      /* 1..TSPH_MAX_PHASES */
    int32_t solver_type;    /* TSPH_DFSPH or TSPH_VFSPH (aliases, sph_obj.py:65-73) */
    int32_t neighb_range;   /* template half-width r: (2r+1)^dim cells */
    float part_size;        /* part_size[1] */
    float kernel_h;         /* kernel_h[1] = 2 * part_size */
    float kernel_h2;        /* kernel_h[2] */
    float kernel_sig;       /* kernel_sig[dim] */
    float lb[3];            /* sim_space_lb */
    int32_t grid_size[3];   /* ceil((rt - lb) / h) per axis */
    int64_t node_num;       /* product of grid_size */
    float gravity[3];
    float viscosity;        /* dynamic_viscosity */
    float phase_rest_density[TSPH_MAX_PHASES];
    float divergence_threshold;
    float compression_threshold;
    int32_t iter_min, iter_max;
    int32_t cs;             /* integer field in the reference */
    float cfl_factor;
    float fbm_diffusion, fbm_convection;
    float surface_tension_gamma;
    int32_t fbm_enabled;    /* run the volume-fraction block, main.py:244-250 */
    int32_t fbm_max_passes; /* cap on its pass loop (the reference has none) */
    int32_t wc_gamma;       /* solver_wc_gamma (integer field, sph_config.py:167) */
    int32_t wcsph_enabled;  /* run the weakly compressible pressure block, main.py:238-242 */
} tsph_params;

/* Views of one particle set: the fields of `Fluid`, sph_obj.py:24-63, in the
 * caller's particle order.  Vectors are [capacity][dim] row-major, volume
 * fractions [capacity][phase_num], drift velocities [capacity][phase_num][dim]. */
typedef struct tsph_set {
    int64_t n;              /* part_num[None] */
    int64_t capacity;       /* max_part_num */
    float *pos, *vel, *vel_adv, *acce, *acce_adv;
    float *mass, *rest_density, *rest_volume;
    float *volume_frac, *volume_frac_tmp;
    float *W, *sph_density, *sph_compression, *psi_adv;
    float *alpha, *alpha_1, *alpha_2;
    float *normal, *drift_vel, *fbm_zeta;
    float *pressure;        /* written by the weakly compressible block (fluid) */
    int32_t *flag;
    int32_t *neighb_cell_seq, *neighb_in_cell_seq, *neighb_cell_structured_seq;
} tsph_set;

/* Host-side copy of the step's scalars (fields `compression`,
 * `statistics_*_energy` of sph_obj.py:41-47, `config.dt`, and the counters of
 * GlobalVariable, sph_obj.py:347-360). */
typedef struct tsph_stats {
    double dt;
    double time_count;
    double compression;
    double kinetic_energy;
    double potential_energy;
    int32_t div_iter;
    int32_t incom_iter;
    int32_t fbm_passes;
    int32_t general_flag;
    int32_t status;
    int32_t fluid_in_grid;
    int32_t bound_in_grid;
    int32_t steps;
    /* cumulative over all steps of this context */
    int64_t total_div_iter;
    int64_t total_incom_iter;
    int64_t total_fbm_passes;
    double max_dens_compression;   /* largest compression left by a density solve */
    int32_t launches_per_step;     /* kernels per step outside the solver / pass loops */
    int32_t launches_per_iter;     /* kernels per solver iteration */
    int32_t launches_per_pass;     /* kernels per volume-fraction pass */
    int32_t pad;
} tsph_stats;

/* Phases timed by tsph_profile_phases, in output order. */
enum {
    TSPH_PH_CFL = 0,        /* cfl_condition */
    TSPH_PH_GRID = 1,       /* cell grid build + gather into sorted order */
    TSPH_PH_DENSITY = 2,    /* density / alpha sweeps (fluid, boundary) */
    TSPH_PH_PSI = 3,        /* Jacobi sweep A: psi_adv and its reduction */
    TSPH_PH_VEL = 4,        /* Jacobi sweep B: v_adv update + loop test */
    TSPH_PH_ADVECT = 5,     /* viscosity, surface tension, v_adv predict */
    TSPH_PH_UNSORT = 6,     /* update + write-back in caller order */
    TSPH_PH_COUNT = 7
};

typedef struct tsph_ctx tsph_ctx;

/* Allocates the solver context: cell grids sized node_num, sorted particle
 * buffers sized by the capacities, reduction scratch.  Replaces Ngrid()
 * (sph_obj.py:281-293) plus the solver fields of Fluid.  Returns TSPH_OK. */
int tsph_create(const tsph_params *params, int64_t fluid_capacity, int64_t bound_capacity,
                tsph_ctx **out);

/* A context that steps n_scenes independent scenes in the same launches (the
 * batched form; the reference runs one scene per process, main.py:8-12).  Scene
 * s has its own parameters (box, grid, rest densities, thresholds ...; dim,
 * phase_num, solver_type, neighb_range and fbm_enabled must be equal) and its own
 * dt, solver loops and iteration counts, as if it ran alone.  Its particles are
 * fluid_counts[s] / bound_counts[s] consecutive entries of the caller's fluid and
 * boundary sets, in scene order; the sets' n must equal the count totals. */
int tsph_create_batch(const tsph_params *scenes, int n_scenes, const int64_t *fluid_counts,
                      const int64_t *bound_counts, tsph_ctx **out);
int tsph_destroy(tsph_ctx *ctx);

/* Selects how the two solver loops run: 1 = one CUDA graph per substep with
 * device-side while nodes (default), 0 = host-driven loops that read the
 * convergence value every iteration like main.py:201,222. */
int tsph_set_graph_mode(tsph_ctx *ctx, int use_graph);

/* Threads per particle of the neighbour-list sweeps (1, 2, 4 or 8; default 1).
 * A tuning knob with no counterpart in the reference: results are the same up to
 * FP32 summation order, and deterministic for a given setting. */
int tsph_set_threads_per_particle(tsph_ctx *ctx, int threads_per_particle);

/* cfl_condition(fluid), sph.py:41-47: dt on the device.  Also adds dt to the
 * device clock, as run_step does on the host (main.py:348-349). */
int tsph_cfl_condition(tsph_ctx *ctx, const tsph_set *fluid, void *stream);

/* sph_step(), main.py:175-256, with the current device dt: grid build,
 * density/alpha, divergence solve, viscosity, surface tension, density solve,
 * volume-fraction update when fbm_enabled, mass/position/energy update. */
int tsph_sph_step(tsph_ctx *ctx, const tsph_set *fluid, const tsph_set *bound, void *stream);

/* One substep of run_step (main.py:348-352): cfl_condition, clock, sph_step. */
int tsph_substep(tsph_ctx *ctx, const tsph_set *fluid, const tsph_set *bound, void *stream);

/* ------------------------------------------------- kernel-level composition
 * sph_step (main.py:175-256) split at the reference's own seams, for callers
 * that compose the step themselves as main.py does from the kernels of
 * sph.py.  One-scene contexts only.  The same kernels as tsph_sph_step run in
 * the same order, so a step composed of these calls in main.py's order equals
 * tsph_sph_step bit for bit.  Between tsph_grid_build and tsph_update the
 * step's state lives in the context in cell order: the caller's arrays are read
 * by tsph_grid_build and written by tsph_update only.  Calls out of order
 * return TSPH_ERR_STATE. */
enum { TSPH_SOLVE_DIV = 0, TSPH_SOLVE_DENS = 1 };
enum {
    TSPH_TERM_GRAVITY = 1,          /* SPH_advection_gravity_acc, sph.py:108-111 */
    TSPH_TERM_VISCOSITY = 2,        /* SPH_advection_viscosity_acc, sph.py:114-129 */
    TSPH_TERM_SURFACE_TENSION = 4,  /* SPH_advection_surface_tension_acc, sph.py:132-166 */
    TSPH_TERM_ALL = 7
};

/* Starts a step: Ngrid.clear_node / encode / mem_shift / fill_node
 * (sph_obj.py:295-323, main.py:178-183), SPH_clean_value (sph.py:22-38,
 * main.py:185-186) and the gather of both sets into cell order with
 * v_adv = vel (SPH_vel_2_vel_adv, sph.py:253-256, main.py:200). */
int tsph_grid_build(tsph_ctx *ctx, const tsph_set *fluid, const tsph_set *bound, void *stream);

/* SPH_prepare_attr (f,f)(f,b)(b,b)(b,f), SPH_prepare_alpha_1 (f,f)(f,b),
 * SPH_prepare_alpha_2 (f,f)(b,f), SPH_prepare_alpha (f)(b): sph.py:50-105 as
 * main.py:188-197 calls them. */
int tsph_density_alpha(tsph_ctx *ctx, void *stream);

/* One Jacobi sweep A of a pressure solve: IPPE_adv_psi_init, IPPE_adv_psi
 * (f,f)(f,b) and IPPE_psi_adv_non_negative (sph.py:196-226; main.py:203-208 or
 * 224-229).  kind: TSPH_SOLVE_DIV before tsph_nonpressure, TSPH_SOLVE_DENS after.
 * If compression_out is not NULL, synchronises and writes fluid.compression,
 * the mean of psi_adv / psi0 over the fluid that the loop test reads. */
int tsph_adv_psi(tsph_ctx *ctx, int kind, double *compression_out, void *stream);

/* Sweep B: IPPE_update_vel_adv (f,f)(f,b), sph.py:229-244 (main.py:209-210 or
 * 230-231); counts one iteration of the solve `kind`. */
int tsph_update_vel_adv(tsph_ctx *ctx, int kind, void *stream);

/* A whole solver loop, main.py:199-214 (kind TSPH_SOLVE_DIV) or 221-234
 * (TSPH_SOLVE_DENS): while it < it_min or compression > tol, one sweep A and
 * one sweep B; stops after it_max + 1 iterations.  tol < 0, it_min < 0 or
 * it_max < 0 take the scene's own value (solver_divergence_threshold or
 * solver_compression_threshold, solver_iter_threshold_min / _max).  Host
 * driven, reading the compression after every sweep A as the reference does;
 * writes the iterations run and the final compression. */
int tsph_solve(tsph_ctx *ctx, int kind, double tol, int32_t it_min, int32_t it_max, int32_t *it_out,
               double *err_out, void *stream);

/* SPH_vel_adv_2_vel, the non-pressure forces selected by `terms`
 * (TSPH_TERM_* bits; surface tension only where the scene's gamma is not 0) and
 * SPH_advection_update_vel_adv: sph.py:108-166, 247-262 as main.py:215-220
 * calls them.  Makes the predicted v_adv the density solve's start. */
int tsph_nonpressure(tsph_ctx *ctx, int32_t terms, void *stream);

/* The weakly compressible pressure block, main.py:238-242: WC_pressure_val,
 * WC_pressure_acce (f,f)(f,b), SPH_advection_update_vel_adv (sph.py:169-193,
 * 247-250).  Needs a context created with wcsph_enabled. */
int tsph_wc_pressure(tsph_ctx *ctx, const tsph_set *bound, void *stream);

/* One pass of the volume-fraction loop, main.py:244-248: SPH_FBM_clean_tmp,
 * SPH_FBM_convect, SPH_FBM_diffuse, SPH_FBM_check_tmp (sph.py:301-372); the
 * first pass of a step also computes the drift velocities.  Synchronises and
 * writes fluid.general_flag (1 while some particle was flagged this pass).  A
 * pass after the loop has ended (general_flag 0, or fbm_max_passes reached)
 * does nothing.  Needs a context created with fbm_enabled. */
int tsph_fbm_pass(tsph_ctx *ctx, int32_t *general_flag_out, void *stream);

/* Ends the step: SPH_update_volume_frac (with fbm_enabled), SPH_update_mass,
 * SPH_update_pos, SPH_update_energy (sph.py:265-286, 375-379; main.py:251-256)
 * and the write-back of every field into the caller's arrays. */
int tsph_update(tsph_ctx *ctx, const tsph_set *fluid, const tsph_set *bound, void *stream);

/* Synchronises `stream` and copies the scalars of the last step (scene 0). */
int tsph_read_stats(tsph_ctx *ctx, tsph_stats *out, void *stream);

/* The same for scenes [first, first + count) of a batch, into out[count]. */
int tsph_read_scene_stats(tsph_ctx *ctx, int first, int count, tsph_stats *out, void *stream);

/* Sets the persistent device scalars of every scene (clock, dt, the carried-over
 * compression that the first divergence-loop test reads, main.py:201). */
int tsph_set_state(tsph_ctx *ctx, double time_count, float dt, double compression, void *stream);

/* Debug / parity: builds the grid for the current positions and writes, per
 * particle in caller order, the number of neighbours with 0 < r < h among the
 * fluid ([0]) and the boundary ([1]) set, and an order-independent 64-bit hash
 * of that neighbour set, as found by the candidate scan that records the
 * step's neighbour pairs (it skips template rows and cells beyond h).  fluid_out: int32[n_f][2] + uint64[n_f]; bound_out the
 * same for the boundary set.  Synchronises. */
int tsph_neighbor_stats(tsph_ctx *ctx, const tsph_set *fluid, const tsph_set *bound,
                        int32_t *fluid_counts, uint64_t *fluid_hash,
                        int32_t *bound_counts, uint64_t *bound_hash, void *stream);

/* Measurement: the number of candidates the density sweep's scan visits per
 * particle (caller order) in the fluid grid ([0]) and the boundary grid ([1]),
 * for the current positions; fluid_counts int32[n_f][2], bound_counts
 * int32[n_b][2].  Synchronises. */
int tsph_candidate_stats(tsph_ctx *ctx, const tsph_set *fluid, const tsph_set *bound,
                         int32_t *fluid_counts, int32_t *bound_counts, void *stream);

/* Measurement: the FP32 FMA rate of the current GPU in TFLOP/s (independent
 * fused multiply-add chains on every SM, an FMA counted as two operations),
 * timed with CUDA events on `stream`; synchronises.  Needs no context. */
int tsph_fp32_fma_peak(double *tflops_out, void *stream);

/* Measurement: runs each phase of a step `reps` times back to back on `stream`
 * and writes its mean duration per launch in milliseconds (CUDA events on that
 * stream) to ms_out[TSPH_PH_COUNT].  The phases leave the particle state as one
 * step would (positions advance once); synchronises. */
int tsph_profile_phases(tsph_ctx *ctx, const tsph_set *fluid, const tsph_set *bound, int reps,
                        float *ms_out, void *stream);

/* Fixed limits of tsph_fluid_density_noalloc's scratch (about 3 MB per GPU). */
#define TSPH_NOALLOC_MAX_CELLS 131072
#define TSPH_NOALLOC_MAX_PARTICLES 65536

/* Fluid density sweep that allocates nothing.  No counterpart in the reference:
 * it exists for callers that cannot allocate device memory where they call in
 * (under a host that pre-plans all device memory, or beside an allocator that
 * owns the device) and so cannot hold a tsph_ctx.
 * From caller-owned device arrays (positions [n][dim], masses, rest volumes of
 * the fluid and boundary sets) it writes W, sph_density and sph_compression of
 * every fluid particle -- the sums sph_step's density sweep forms from the same
 * positions.  Working memory is one fixed device array shared by all calls:
 * node_num <= TSPH_NOALLOC_MAX_CELLS and n <= TSPH_NOALLOC_MAX_PARTICLES per set,
 * larger inputs return TSPH_ERR_CAPACITY; calls that overlap on the GPU race.
 * The first call on a device looks the array up in the device's primary
 * context and caches the address (make it before any stream capture; a later
 * cudaDeviceReset or a non-primary context is not supported).
 * Stream-ordered; does not synchronise. */
int tsph_fluid_density_noalloc(const tsph_params *params, const float *fluid_pos, const float *fluid_mass,
                               const float *fluid_rest_volume, int64_t n_fluid, const float *bound_pos,
                               const float *bound_mass, const float *bound_rest_volume, int64_t n_bound,
                               float *W, float *sph_density, float *sph_compression, void *stream);

/* Particle-to-grid velocity map, map_velocity (sph.py:382-397; called at the
 * end of sph_step, main.py:254): for every node I of a regular grid with
 * positions lb + I * dist (shape[0..dim-1], C order) writes
 * grid_vel[I] = sum_j X_j / psi_j * vel_j * W(|pos_I - pos_j|) over the fluid
 * particles of the template cells around the node's cell.  As in the
 * reference the candidates come from the cell grid of the last step (built at
 * its start) and positions / velocities / X / psi are the set's current
 * values.  Call after a step; grid_vel is [prod(shape)][dim] device FP32. */
int tsph_map_velocity(tsph_ctx *ctx, const tsph_set *fluid, const float *lb, float dist, const int32_t *shape,
                      float *grid_vel, void *stream);

/* ---------------------------------------------------------------- adjoint
 * Hand-written reverse mode of the substep (no counterpart in the reference,
 * which has no autodiff; the forward it reverses is tsph_substep, i.e. the
 * substep of main.py:347-352 around sph_step, main.py:175-256).  Supported for
 * a single-scene DFSPH context (viscosity and surface tension; not the
 * volume-fraction update).  Differentiable inputs: fluid positions and velocities at the start
 * of the substep and the dynamic viscosity.  Held fixed: masses, rest
 * densities, the boundary, dt, the iteration counts of the two Jacobi solves
 * (those the forward took) and the neighbour pairs and template candidates of
 * the substep (the topology found at its start).  The clamps psi_adv = max(., 0) and
 * alpha = max(., 1e-4) are differentiated one-sided.
 *
 * A tape holds `slots` recorded substeps (or density evaluations) with at most
 * `max_iters` iterations per Jacobi solve.  Recording writes what the reverse
 * sweeps need -- the sorted order, positions, neighbour lists, density and
 * alpha terms, every Jacobi iterate, and with surface tension the normals and
 * cell starts -- into device memory owned by the tape;
 * the reverse pass reads only the tape.  The caller arranges checkpointing. */
typedef struct tsph_tape tsph_tape;

enum {
    TSPH_TAPE_ITER_OVERFLOW = 1,   /* a solve ran more than max_iters iterations */
    TSPH_TAPE_LIST_OVERFLOW = 2,   /* a particle had more neighbours than its list holds */
    TSPH_TAPE_OUTSIDE_GRID = 4,    /* a fluid particle had no valid cell (one-sided pairs) */
    TSPH_TAPE_BOUND_PSI = 8        /* the boundary's psi_adv was nonzero */
};

int tsph_tape_create(tsph_ctx *ctx, int slots, int max_iters, tsph_tape **out);
int tsph_tape_destroy(tsph_tape *tape);

/* tsph_substep that also records into tape slot `slot`. */
int tsph_substep_record(tsph_ctx *ctx, const tsph_set *fluid, const tsph_set *bound, tsph_tape *tape, int slot,
                        void *stream);

/* Density of every fluid particle at the current positions (the grid build
 * and density sweep of sph_step, sph.py:50-64), written to sph_density_out
 * (caller order, device) and recorded into tape slot `slot`.  Changes no
 * particle field. */
int tsph_density_record(tsph_ctx *ctx, const tsph_set *fluid, const tsph_set *bound, tsph_tape *tape, int slot,
                        float *sph_density_out, void *stream);

/* Reverse of the substep recorded in `slot`: from dL/dpos and dL/dvel after it
 * (caller order, [n][dim], device FP32) writes dL/dpos and dL/dvel before it
 * (may alias the inputs) and adds dL/dviscosity to *grad_viscosity (one
 * device double).  Synchronises once per tape recording to read the slots'
 * iteration counts; returns TSPH_ERR_STATE with the slot's TSPH_TAPE_* bits in
 * the error text when the recording cannot be reversed. */
int tsph_substep_adjoint(tsph_ctx *ctx, tsph_tape *tape, int slot, const float *grad_pos_out,
                         const float *grad_vel_out, float *grad_pos_in, float *grad_vel_in, double *grad_viscosity,
                         void *stream);

/* Reverse of the density evaluation recorded in `slot`: adds dL/dpos to
 * grad_pos ([n][dim]) from dL/dsph_density ([n]); caller order, device. */
int tsph_density_adjoint(tsph_ctx *ctx, tsph_tape *tape, int slot, const float *grad_density, float *grad_pos,
                         void *stream);

/* Sets the dynamic viscosity of scene `scene` (global_dynamic_viscosity,
 * sph_config.py:149) for the following steps. */
int tsph_set_viscosity(tsph_ctx *ctx, int scene, float viscosity);

/* Library version string. */
const char *tsph_version(void);

/* Text of the last error returned on the calling thread ("" if none). */
const char *tsph_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* TICHI_SPH_H */
