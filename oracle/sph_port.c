/*
 * C restatement of Tichi_SPH's per-substep path -- TEST INFRASTRUCTURE ONLY.
 *
 * The checker and the timed CPU baseline, never the product: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.  It follows
 * the reference's own structure kernel by kernel: the combined counting-sort grid
 * with (pid, uid) slots (Ngrid, sph_obj.py:280-323), one parallel loop per Taichi
 * kernel of sph.py, each pair kernel scanning the (2r+1)^d template cells and
 * filtering by uid (sph.py:52-60), and the host-driven solver loops of
 * main.py:175-256.  REAL is float (the reference's default_fp=f32; the CPU
 * baseline) or double (the FP64 oracle: every field, sum and pair term in
 * double; the FP32 particle arrays are converted to double working arrays at
 * the start of a substep and back at its end).  OpenMP parallelises the
 * outermost particle loop of every kernel, as Taichi's CPU backend does, but
 * for the cell fill and the solvers' compression sum, which run serially so
 * that every run of the restatement gives the same bits.
 */
#include <math.h>
#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include <stdlib.h>
#include <string.h>

#include "../include/tichi_sph.h"

#ifndef REAL
#define REAL float
#endif

typedef struct {
    tsph_params p;
    int64_t cap;  /* fluid + bound capacity */
    int32_t *node_part_count, *node_part_shift, *node_part_shift_count;
    int32_t *part_pid_in_node, *part_uid_in_node;
    int32_t *tmpl; /* [ntmpl][dim] */
    int ntmpl;
    REAL dt;
    REAL compression;
    double time_count;
} port_ctx;

typedef struct {
    double dt, time_count, compression, kinetic_energy, potential_energy;
    int32_t div_iter, incom_iter, fbm_passes;
} port_stats;

/* the fields of one particle set (the tsph_set fields) in REAL */
typedef struct {
    int64_t n;
    REAL *pos, *vel, *vel_adv, *acce, *acce_adv;
    REAL *mass, *rest_density, *rest_volume;
    REAL *volume_frac, *volume_frac_tmp;
    REAL *W, *sph_density, *sph_compression, *psi_adv;
    REAL *alpha, *alpha_1, *alpha_2;
    REAL *normal, *drift_vel, *fbm_zeta;
    REAL *pressure;
    int32_t *flag;
    int32_t *neighb_cell_seq, *neighb_in_cell_seq, *neighb_cell_structured_seq;
} rset;

/* one particle set: its fields + uid and the solver aliases */
typedef struct {
    rset *s;
    int uid;
    REAL *X, *psi; /* X = mass | rest_volume; sph_psi = sph_density | sph_compression */
    REAL *rest_psi; /* NULL means the `ones` field (VFSPH) */
    double compression, ke, pe;
    int general_flag;
} obj_t;

#define D (c->p.dim)
#define P (c->p.phase_num)

static REAL kW(const port_ctx *c, REAL r) {
    REAL q = r / (REAL)c->p.kernel_h, t = 0;
    if (q <= (REAL)0.5) t = 6 * (q * q * q - q * q) + 1;
    else if (q < 1) t = 2 * (1 - q) * (1 - q) * (1 - q);
    return t * (REAL)c->p.kernel_sig;
}
static REAL kWg(const port_ctx *c, REAL r) {
    REAL q = r / (REAL)c->p.kernel_h, t = 0;
    if (q <= (REAL)0.5) t = 6 * (3 * q * q - 2 * q);
    else if (q < 1) t = -6 * (1 - q) * (1 - q);
    return t * ((REAL)c->p.kernel_sig / (REAL)c->p.kernel_h);
}
static REAL kC(const port_ctx *c, REAL r) {
    REAL h = (REAL)c->p.kernel_h, q = r / h, t = 0;
    if (q <= (REAL)0.5) t = 2 * (1 - q) * (1 - q) * (1 - q) * q * q * q - (REAL)1 / 64;
    else if (q < 1) t = (1 - q) * (1 - q) * (1 - q) * q * q * q;
    return t * ((REAL)32 / (REAL)3.14159265358979323846 / (h * h * h));
}
static REAL rest_psi(const obj_t *o, int64_t i) { return o->rest_psi ? (REAL)o->rest_psi[i] : (REAL)1; }
static int64_t code_of(const port_ctx *c, const int32_t *st) {
    int64_t code = 0, coder = 1;
    for (int d = 0; d < D; ++d) {
        code += (int64_t)st[d] * coder;
        coder *= c->p.grid_size[d];
    }
    return code;
}

/* ---------------------------------------------------------------- Ngrid */
static void clear_node(port_ctx *c) { memset(c->node_part_count, 0, sizeof(int32_t) * c->p.node_num); }

static void encode(port_ctx *c, obj_t *o) {
    rset *s = o->s;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < s->n; ++i) {
        for (int d = 0; d < D; ++d) {
            float f = floorf(((float)s->pos[i * D + d] - c->p.lb[d]) / c->p.kernel_h);
            s->neighb_cell_structured_seq[i * D + d] = (int32_t)f;
        }
        int64_t code = code_of(c, s->neighb_cell_structured_seq + i * D);
        s->neighb_cell_seq[i] = (int32_t)code;
        if (0 < code && code < c->p.node_num) {
#pragma omp atomic
            c->node_part_count[code] += 1;
        }
    }
}

static void mem_shift(port_ctx *c) {
    int32_t sum = 0;
    for (int64_t i = 0; i < c->p.node_num; ++i) {
        c->node_part_shift[i] = sum;
        c->node_part_shift_count[i] = sum;
        sum += c->node_part_count[i];
    }
}

/* The reference fills a cell through an atomic counter (any order of its
 * particles is valid); this fill runs serially, so each cell holds its
 * particles in id order on every run, as the CUDA path's cells do: the
 * restatement's sums then run in one fixed order. */
static void fill_node(port_ctx *c, obj_t *o) {
    rset *s = o->s;
    for (int64_t i = 0; i < s->n; ++i) {
        int32_t code = s->neighb_cell_seq[i];
        if (0 < code && code < c->p.node_num) {
            int32_t slot = c->node_part_shift_count[code]++;
            s->neighb_in_cell_seq[i] = slot;
            c->part_pid_in_node[slot] = (int32_t)i;
            c->part_uid_in_node[slot] = o->uid;
        }
    }
}

/* The reference's neighbour-loop template (sph.py:9-19): for particle i of obj,
 * every j of nobj found in the template cells; the body sees i, j. */
#define FOR_NEIGHBOURS(c, o, no, i, j, ...)                                           \
    do {                                                                               \
        int32_t st_[3];                                                                \
        for (int t_ = 0; t_ < (c)->ntmpl; ++t_) {                                      \
            for (int d_ = 0; d_ < D; ++d_)                                             \
                st_[d_] = (o)->s->neighb_cell_structured_seq[(i) * D + d_] + (c)->tmpl[t_ * D + d_]; \
            int64_t nc_ = code_of((c), st_);                                           \
            if (0 < nc_ && nc_ < (c)->p.node_num) {                                    \
                int32_t cnt_ = (c)->node_part_count[nc_], sh_ = (c)->node_part_shift[nc_]; \
                for (int32_t k_ = 0; k_ < cnt_; ++k_) {                                \
                    if ((c)->part_uid_in_node[sh_ + k_] == (no)->uid) {                \
                        int64_t j = (c)->part_pid_in_node[sh_ + k_];                   \
                        __VA_ARGS__                                                    \
                    }                                                                  \
                }                                                                      \
            }                                                                          \
        }                                                                              \
    } while (0)

#define XIJ(o, no, i, j, x, r)                                                         \
    REAL x[3] = {0, 0, 0};                                                             \
    for (int d_ = 0; d_ < D; ++d_) x[d_] = (REAL)(o)->s->pos[(i) * D + d_] - (REAL)(no)->s->pos[(j) * D + d_]; \
    REAL r = (REAL)sqrt((double)(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]))

/* ---------------------------------------------------------------- sph.py */
static void clean_value(port_ctx *c, obj_t *o) {
    rset *s = o->s;
    o->general_flag = 1;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < s->n; ++i) {
        s->W[i] = 0; s->sph_compression[i] = 0; s->sph_density[i] = 0; s->alpha_2[i] = 0; s->flag[i] = 0;
        for (int d = 0; d < D; ++d) {
            s->acce[i * D + d] = 0; s->acce_adv[i * D + d] = 0; s->alpha_1[i * D + d] = 0;
            for (int k = 0; k < P; ++k) s->drift_vel[(i * P + k) * D + d] = 0;
        }
    }
}

static void cfl_condition(port_ctx *c, obj_t *o) {
    REAL dt = (REAL)c->p.part_size / (REAL)c->p.cs;
    rset *s = o->s;
    for (int64_t i = 0; i < s->n; ++i) {
        REAL v2 = 0;
        for (int d = 0; d < D; ++d) v2 += (REAL)s->vel[i * D + d] * (REAL)s->vel[i * D + d];
        REAL vn = (REAL)sqrt((double)v2);
        if (vn > (REAL)1e-4) {
            REAL t = (REAL)c->p.part_size / vn * (REAL)c->p.cfl_factor;
            if (t < dt) dt = t;
        }
    }
    /* config.dt is an f32 field in the reference (sph_config.py:100): the FP64
     * build rounds it there too */
    c->dt = (REAL)(float)dt;
}

static void prepare_attr(port_ctx *c, obj_t *o, obj_t *no) {
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < o->s->n; ++i) {
        REAL w = 0, sc = 0, sd = 0;
        FOR_NEIGHBOURS(c, o, no, i, j, {
            XIJ(o, no, i, j, x, r);
            REAL Wr = kW(c, r);
            w += Wr; sc += Wr * no->s->rest_volume[j]; sd += Wr * no->s->mass[j];
        });
        o->s->W[i] += w; o->s->sph_compression[i] += sc; o->s->sph_density[i] += sd;
    }
}

static void prepare_alpha_1(port_ctx *c, obj_t *o, obj_t *no) {
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < o->s->n; ++i) {
        REAL a[3] = {0, 0, 0};
        FOR_NEIGHBOURS(c, o, no, i, j, {
            XIJ(o, no, i, j, x, r);
            if (r > 0) {
                REAL f = no->X[j] * kWg(c, r) / r;
                for (int d = 0; d < D; ++d) a[d] += f * x[d];
            }
        });
        for (int d = 0; d < D; ++d) o->s->alpha_1[i * D + d] += a[d];
    }
}

static void prepare_alpha_2(port_ctx *c, obj_t *o, obj_t *no) {
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < o->s->n; ++i) {
        REAL a = 0;
        FOR_NEIGHBOURS(c, o, no, i, j, {
            XIJ(o, no, i, j, x, r);
            if (r > 0) {
                REAL g = kWg(c, r);
                a += g * g * no->X[j] * no->X[j] / no->s->mass[j];
            }
        });
        o->s->alpha_2[i] += a;
    }
}

static void prepare_alpha(port_ctx *c, obj_t *o) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < o->s->n; ++i) {
        REAL a = 0;
        for (int d = 0; d < D; ++d) a += (REAL)o->s->alpha_1[i * D + d] * o->s->alpha_1[i * D + d];
        a = a / o->s->mass[i] + o->s->alpha_2[i];
        o->s->alpha[i] = a < (REAL)1e-4 ? (REAL)1e-4 : a;
    }
}

static void gravity_acc(port_ctx *c, obj_t *o) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < o->s->n; ++i)
        for (int d = 0; d < D; ++d) o->s->acce_adv[i * D + d] += c->p.gravity[d];
}

static void viscosity_acc(port_ctx *c, obj_t *o, obj_t *no) {
    const REAL h2 = (REAL)c->p.kernel_h2;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < o->s->n; ++i) {
        REAL a[3] = {0, 0, 0};
        REAL s = (REAL)c->p.viscosity / o->s->rest_density[i];
        FOR_NEIGHBOURS(c, o, no, i, j, {
            XIJ(o, no, i, j, x, r);
            if (r > 0) {
                REAL Vj = no->X[j] / no->psi[j];
                REAL Ax = 0;
                for (int d = 0; d < D; ++d) Ax += ((REAL)o->s->vel[i * D + d] - no->s->vel[j * D + d]) * x[d];
                REAL f = 2 * (2 + D) * Vj * kWg(c, r) * Ax / ((REAL)0.01 * h2 + r * r) / r;
                for (int d = 0; d < D; ++d) a[d] += f * x[d] * s;
            }
        });
        for (int d = 0; d < D; ++d) o->s->acce_adv[i * D + d] += a[d];
    }
}

static void surface_tension_acc(port_ctx *c, obj_t *o, obj_t *no) {
    const REAL gam = (REAL)c->p.surface_tension_gamma, h = (REAL)c->p.kernel_h;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < o->s->n; ++i) {
        REAL nv[3] = {0, 0, 0};
        FOR_NEIGHBOURS(c, o, no, i, j, {
            XIJ(o, no, i, j, x, r);
            if (r > 0) {
                REAL f = -no->X[j] / no->psi[j] * kWg(c, r) / r;
                for (int d = 0; d < D; ++d) nv[d] += f * x[d];
            }
        });
        for (int d = 0; d < D; ++d) o->s->normal[i * D + d] = nv[d] * h;
    }
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < o->s->n; ++i) {
        REAL a[3] = {0, 0, 0};
        FOR_NEIGHBOURS(c, o, no, i, j, {
            XIJ(o, no, i, j, x, r);
            /* sph.py:163 compares an f32 field with a literal that Taichi's default_fp=f32
             * makes 0.99f; both builds compare the stored f32 values with 0.99f */
            if (r > 0 && o->s->volume_frac[i * P] > 0.99f && no->s->volume_frac[j * P] > 0.99f) {
                REAL coh = -gam * no->s->mass[j] * kC(c, r) / r;
                REAL fac = 2 * rest_psi(o, i) / (o->psi[i] + no->psi[j]);
                for (int d = 0; d < D; ++d)
                    a[d] += fac * (coh * x[d] + gam * ((REAL)o->s->normal[i * D + d] - no->s->normal[j * D + d]));
            }
        });
        for (int d = 0; d < D; ++d) o->s->acce_adv[i * D + d] += a[d];
    }
}

static void adv_psi_init(port_ctx *c, obj_t *o) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < o->s->n; ++i) o->s->psi_adv[i] = o->psi[i] - rest_psi(o, i);
}

static void adv_psi(port_ctx *c, obj_t *o, obj_t *no) {
    const REAL dt = c->dt;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < o->s->n; ++i) {
        REAL acc = 0;
        FOR_NEIGHBOURS(c, o, no, i, j, {
            XIJ(o, no, i, j, x, r);
            if (r > 0) {
                REAL g = kWg(c, r) / r, dv = 0;
                for (int d = 0; d < D; ++d) dv += x[d] * ((REAL)o->s->vel_adv[i * D + d] - no->s->vel_adv[j * D + d]);
                acc += g * dv * no->X[j] * dt;
            }
        });
        o->s->psi_adv[i] += acc;
    }
}

/* The sum runs serially in id order: an OpenMP reduction combines the threads'
 * partial sums in no fixed order, and the solver loops branch on this value. */
static void psi_adv_non_negative(port_ctx *c, obj_t *o) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < o->s->n; ++i)
        if (o->s->psi_adv[i] < 0) o->s->psi_adv[i] = 0;
    REAL sum = 0;
    for (int64_t i = 0; i < o->s->n; ++i) sum += o->s->psi_adv[i] / rest_psi(o, i);
    c->compression = sum / (REAL)o->s->n;
}

static void update_vel_adv(port_ctx *c, obj_t *o, obj_t *no) {
    const REAL dt = c->dt;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < o->s->n; ++i) {
        REAL a[3] = {0, 0, 0};
        FOR_NEIGHBOURS(c, o, no, i, j, {
            XIJ(o, no, i, j, x, r);
            if (r > 0) {
                REAL coef = o->s->psi_adv[i] * no->X[j] / o->s->alpha[i] + no->s->psi_adv[j] * o->X[i] / no->s->alpha[j];
                REAL f = -(1 / dt) * coef * kWg(c, r) / r / o->s->mass[i];
                for (int d = 0; d < D; ++d) a[d] += f * x[d];
            }
        });
        for (int d = 0; d < D; ++d) o->s->vel_adv[i * D + d] += a[d];
    }
}

static void fbm_convect(port_ctx *c, obj_t *o, obj_t *no) {
    const REAL dt = c->dt;
    rset *s = o->s;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < s->n; ++i) {
        REAL zeta = 0;
        for (int d = 0; d < D; ++d) s->acce_adv[i * D + d] = ((REAL)s->vel_adv[i * D + d] - s->vel[i * D + d]) / dt;
        for (int k = 0; k < P; ++k) {
            REAL rk = c->p.phase_rest_density[k];
            zeta += s->volume_frac[i * P + k] * (rk - s->rest_density[i]) / rk;
        }
        s->fbm_zeta[i] = zeta;
        for (int d = 0; d < D; ++d) s->acce[i * D + d] = ((REAL)s->acce_adv[i * D + d] - zeta * c->p.gravity[d]) / (1 - zeta);
        for (int k = 0; k < P; ++k) {
            REAL rk = c->p.phase_rest_density[k], vf = s->volume_frac[i * P + k];
            REAL w = vf * rk;
            for (int d = 0; d < D; ++d) {
                REAL dv = vf * (rk - s->rest_density[i]) * ((REAL)c->p.gravity[d] - s->acce[i * D + d]);
                dv = w > (REAL)1e-6 ? dv / w : dv * 0;
                dv += (REAL)s->acce[i * D + d] - s->acce_adv[i * D + d];
                s->drift_vel[(i * P + k) * D + d] = dv * dt;
            }
        }
    }
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < s->n; ++i) {
        if (s->flag[i] != 0) continue;
        REAL t[TSPH_MAX_PHASES] = {0};
        FOR_NEIGHBOURS(c, o, no, i, j, {
            if (no->s->flag[j] == 0) {
                XIJ(o, no, i, j, x, r);
                if (r > 0) {
                    REAL g = kWg(c, r) / r;
                    for (int k = 0; k < P; ++k) {
                        REAL dot = 0;
                        for (int d = 0; d < D; ++d)
                            dot += ((REAL)s->volume_frac[i * P + k] * s->drift_vel[(i * P + k) * D + d] +
                                    (REAL)no->s->volume_frac[j * P + k] * no->s->drift_vel[(j * P + k) * D + d]) * x[d] * g;
                        t[k] -= (REAL)c->p.fbm_convection * dt * no->s->rest_volume[j] * dot;
                    }
                }
            }
        });
        for (int k = 0; k < P; ++k) s->volume_frac_tmp[i * P + k] += t[k];
    }
}

static void fbm_diffuse(port_ctx *c, obj_t *o, obj_t *no) {
    const REAL dt = c->dt, h2 = (REAL)c->p.kernel_h2;
    rset *s = o->s;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < s->n; ++i) {
        if (s->flag[i] != 0) continue;
        REAL t[TSPH_MAX_PHASES] = {0};
        FOR_NEIGHBOURS(c, o, no, i, j, {
            if (no->s->flag[j] == 0) {
                XIJ(o, no, i, j, x, r);
                if (r > 0) {
                    REAL w = dt * (REAL)c->p.fbm_diffusion * no->s->rest_volume[j] * r * kWg(c, r) / (r * r + (REAL)0.01 * h2);
                    for (int k = 0; k < P; ++k) t[k] += ((REAL)s->volume_frac[i * P + k] - no->s->volume_frac[j * P + k]) * w;
                }
            }
        });
        for (int k = 0; k < P; ++k) s->volume_frac_tmp[i * P + k] += t[k];
    }
}

static int fbm_check_tmp(port_ctx *c, obj_t *o) {
    int gf = 0;
    rset *s = o->s;
#pragma omp parallel for schedule(static) reduction(| : gf)
    for (int64_t i = 0; i < s->n; ++i) {
        int neg = 0;
        for (int k = 0; k < P; ++k)
            if ((REAL)s->volume_frac[i * P + k] + s->volume_frac_tmp[i * P + k] < 0) neg = 1;
        if (neg) { s->flag[i] = 1; gf = 1; }
    }
    o->general_flag = gf;
    return gf;
}

static void update_tail(port_ctx *c, obj_t *o, int fbm) {
    rset *s = o->s;
    const REAL dt = c->dt;
    double ke = 0, pe = 0;
#pragma omp parallel for schedule(static) reduction(+ : ke, pe)
    for (int64_t i = 0; i < s->n; ++i) {
        if (fbm && !(s->flag[i] > 0))
            for (int k = 0; k < P; ++k) s->volume_frac[i * P + k] += s->volume_frac_tmp[i * P + k];
        REAL rho = 0;
        for (int k = 0; k < P; ++k) rho += (REAL)c->p.phase_rest_density[k] * s->volume_frac[i * P + k];
        s->rest_density[i] = rho;
        s->mass[i] = rho * s->rest_volume[i];
        REAL v2 = 0;
        for (int d = 0; d < D; ++d) {
            s->vel[i * D + d] = s->vel_adv[i * D + d];
            s->pos[i * D + d] += s->vel[i * D + d] * dt;
            v2 += (REAL)s->vel[i * D + d] * s->vel[i * D + d];
        }
        ke += (REAL)0.5 * s->mass[i] * v2;
        pe += -s->mass[i] * c->p.gravity[1] * (s->pos[i * D + 1] - c->p.lb[1]);
    }
    o->ke = ke;
    o->pe = pe;
}

static int solve(port_ctx *c, obj_t *f, obj_t *b, REAL tol) {
    int it = 0;
    while (it < c->p.iter_min || c->compression > tol) {
        adv_psi_init(c, f);
        adv_psi(c, f, f);
        adv_psi(c, f, b);
        psi_adv_non_negative(c, f);
        update_vel_adv(c, f, f);
        update_vel_adv(c, f, b);
        ++it;
        if (it > c->p.iter_max) break;
    }
    return it;
}

static void bind(port_ctx *c, obj_t *o, rset *s, int uid) {
    memset(o, 0, sizeof(*o));
    o->s = s;
    o->uid = uid;
    int vf = c->p.solver_type == TSPH_VFSPH;
    o->X = vf ? s->rest_volume : s->mass;
    o->psi = vf ? s->sph_compression : s->sph_density;
    o->rest_psi = vf ? NULL : s->rest_density;
}

/* ---------------------------------------------------------------- API */
void *port_create(const tsph_params *p, int64_t capf, int64_t capb) {
    port_ctx *c = (port_ctx *)calloc(1, sizeof(port_ctx));
    c->p = *p;
    c->cap = capf + capb;
    c->node_part_count = (int32_t *)calloc(p->node_num, sizeof(int32_t));
    c->node_part_shift = (int32_t *)calloc(p->node_num, sizeof(int32_t));
    c->node_part_shift_count = (int32_t *)calloc(p->node_num, sizeof(int32_t));
    c->part_pid_in_node = (int32_t *)calloc(c->cap + 1, sizeof(int32_t));
    c->part_uid_in_node = (int32_t *)calloc(c->cap + 1, sizeof(int32_t));
    int w = 2 * p->neighb_range + 1, n = 1;
    for (int d = 0; d < p->dim; ++d) n *= w;
    c->ntmpl = n;
    c->tmpl = (int32_t *)calloc((size_t)n * (size_t)(p->dim > 0 ? p->dim : 1), sizeof(int32_t));
    for (int j = 0; j < n; ++j) {  /* sph_config.py:220-224 */
        int tmp = j;
        for (int d = 0; d < p->dim; ++d) {
            int pw = 1;
            for (int e = 0; e < p->dim - d - 1; ++e) pw *= w;
            int digit = tmp / pw;
            tmp = tmp % pw;
            c->tmpl[j * p->dim + (p->dim - d - 1)] = -p->neighb_range + digit;
        }
    }
    return c;
}

void port_destroy(void *h) {
    port_ctx *c = (port_ctx *)h;
    if (!c) return;
    free(c->node_part_count); free(c->node_part_shift); free(c->node_part_shift_count);
    free(c->part_pid_in_node); free(c->part_uid_in_node); free(c->tmpl);
    free(c);
}

void port_set_state(void *h, double time_count, double compression) {
    port_ctx *c = (port_ctx *)h;
    c->time_count = time_count;
    c->compression = (REAL)compression;
}

/* run_step's substep (main.py:347-352) around sph_step (main.py:175-256). */
/* The REAL view of a tsph_set: its own arrays when REAL is float, else double
 * copies of every field (the number of components of each: 1, dim, phases or
 * phases x dim). */
#define RSET_FIELDS(X_)                                                                          \
    X_(pos, D) X_(vel, D) X_(vel_adv, D) X_(acce, D) X_(acce_adv, D) X_(mass, 1) X_(rest_density, 1) \
    X_(rest_volume, 1) X_(volume_frac, P) X_(volume_frac_tmp, P) X_(W, 1) X_(sph_density, 1)       \
    X_(sph_compression, 1) X_(psi_adv, 1) X_(alpha, 1) X_(alpha_1, D) X_(alpha_2, 1) X_(normal, D)  \
    X_(drift_vel, P * D) X_(fbm_zeta, 1) X_(pressure, 1)

static void rset_in(const port_ctx *c, rset *r, const tsph_set *t) {
    r->n = t->n;
    r->flag = t->flag;
    r->neighb_cell_seq = t->neighb_cell_seq;
    r->neighb_in_cell_seq = t->neighb_in_cell_seq;
    r->neighb_cell_structured_seq = t->neighb_cell_structured_seq;
    const int64_t n = t->n > 0 ? t->n : 1;
#define RSET_IN(f, k)                                                                   \
    if (sizeof(REAL) == sizeof(float)) {                                                \
        r->f = (REAL *)t->f;                                                            \
    } else {                                                                            \
        r->f = (REAL *)malloc(sizeof(REAL) * (size_t)(n * (k)));                        \
        for (int64_t i = 0; i < t->n * (k); ++i) r->f[i] = (REAL)t->f[i];              \
    }
    RSET_FIELDS(RSET_IN)
#undef RSET_IN
}

static void rset_out(const port_ctx *c, rset *r, tsph_set *t) {
    if (sizeof(REAL) == sizeof(float)) return;
#define RSET_OUT(f, k)                                                         \
    for (int64_t i = 0; i < t->n * (k); ++i) t->f[i] = (float)r->f[i];       \
    free(r->f);
    RSET_FIELDS(RSET_OUT)
#undef RSET_OUT
}

int port_substep(void *h, tsph_set *fluid_set, tsph_set *bound_set, port_stats *out) {
    port_ctx *c = (port_ctx *)h;
    rset fr, br;
    rset_in(c, &fr, fluid_set);
    rset_in(c, &br, bound_set);
    rset *fluid = &fr, *bound = &br;
    obj_t F, B;
    bind(c, &F, fluid, 0);
    bind(c, &B, bound, 1);
    cfl_condition(c, &F);
    c->time_count += (double)c->dt;
    clear_node(c);
    encode(c, &F); encode(c, &B);
    mem_shift(c);
    fill_node(c, &F); fill_node(c, &B);
    clean_value(c, &F); clean_value(c, &B);
    prepare_attr(c, &F, &F); prepare_attr(c, &F, &B); prepare_attr(c, &B, &B); prepare_attr(c, &B, &F);
    prepare_alpha_1(c, &F, &F); prepare_alpha_1(c, &F, &B);
    prepare_alpha_2(c, &F, &F); prepare_alpha_2(c, &B, &F);
    prepare_alpha(c, &F); prepare_alpha(c, &B);
    memcpy(fluid->vel_adv, fluid->vel, sizeof(REAL) * fluid->n * D);
    int kd = solve(c, &F, &B, (REAL)c->p.divergence_threshold);
    memcpy(fluid->vel, fluid->vel_adv, sizeof(REAL) * fluid->n * D);
    gravity_acc(c, &F);
    viscosity_acc(c, &F, &F);
    surface_tension_acc(c, &F, &F);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < fluid->n * D; ++i) fluid->vel_adv[i] = fluid->vel[i] + fluid->acce_adv[i] * c->dt;
    int kp = solve(c, &F, &B, (REAL)c->p.compression_threshold);
    int passes = 0;
    if (c->p.fbm_enabled) {
        F.general_flag = 1;
        while (F.general_flag > 0) {
            memset(fluid->volume_frac_tmp, 0, sizeof(REAL) * fluid->n * P);
            fbm_convect(c, &F, &F);
            fbm_diffuse(c, &F, &F);
            fbm_check_tmp(c, &F);
            ++passes;
            if (c->p.fbm_max_passes > 0 && passes >= c->p.fbm_max_passes) break;
        }
    }
    update_tail(c, &F, c->p.fbm_enabled);
    rset_out(c, &fr, fluid_set);
    rset_out(c, &br, bound_set);
    if (out) {
        out->dt = c->dt;
        out->time_count = c->time_count;
        out->compression = c->compression;
        out->kinetic_energy = F.ke;
        out->potential_energy = F.pe;
        out->div_iter = kd;
        out->incom_iter = kp;
        out->fbm_passes = passes;
    }
    return 0;
}

int port_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
