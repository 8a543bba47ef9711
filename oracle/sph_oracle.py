"""FP64 CPU oracle of Tichi_SPH's per-substep hot path.  TEST INFRASTRUCTURE ONLY.

This module is the checker, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may import it.
It restates, in vectorised numpy, the reference kernels in ``sph.py``,
``sph_util.py`` and ``sph_obj.py`` and the step composition of ``main.py``; each
function cites the reference line it follows.  Its parity is pinned by
``tests/test_oracle_golden.py`` against golden vectors recorded by running the
reference's own kernel code (``tests/golden/make_golden.py``): with the same
inputs they agree to ~1e-12 relative, and the iteration counts are identical.

Conventions
-----------
* All arithmetic is float64.  ``Params.from_config(..., taichi_f32=True)`` rounds
  every config scalar the way the reference's f32 Taichi fields store it, which is
  what the CUDA path uses.
* Neighbour candidates are enumerated exactly as the reference does
  (``sph.py:52-60``): the (2r+1)^d template around the particle's cell, linear
  cell codes ``x + nx*y + nx*ny*z`` with no per-axis bounds check (so an x offset
  past a row end wraps into the next row) and a cell is searched iff
  ``0 < code < node_num``.  Particles whose own code is outside that range are
  not in the grid (``sph_obj.py:305,319``).
"""
import json
import math

import numpy as np

F32 = np.float32


# ----------------------------------------------------------------------------- params
class Params:
    """Solver constants; mirrors ``Config`` in ``sph_config.py:83-235``."""

    @classmethod
    def from_files(cls, config_path, scenario_path, taichi_f32=False):
        with open(config_path) as f:
            cfg = json.load(f)
        with open(scenario_path) as f:
            scen = json.load(f)
        return cls.from_config(cfg, scen, taichi_f32=taichi_f32)

    @classmethod
    def from_config(cls, cfg, scen, taichi_f32=False):
        p = cls()
        env = scen["sim_env"]
        rnd = (lambda x: float(F32(x))) if taichi_f32 else (lambda x: float(x))
        p.dim = int(env["sim_dim"])
        p.phase_num = int(env["phase_num"])
        p.solver_type = cfg["solver_type"]
        p.neighb_range = int(cfg["solver_neighb_range"])
        # sph_config.py:145-163
        p.part_size = rnd(env["global_part_size"])
        p.part_size_pow = [1.0, p.part_size, rnd(p.part_size ** 2), rnd(p.part_size ** 3)]
        p.viscosity = rnd(env["global_dynamic_viscosity"])
        p.lb = np.array([rnd(x) for x in env["sim_space_lb"]], dtype=np.float64)
        p.rt = np.array([rnd(x) for x in env["sim_space_rt"]], dtype=np.float64)
        p.gravity = np.array([rnd(x) for x in env["gravity"]], dtype=np.float64)
        p.phase_rest_density = np.array([rnd(x) for x in env["phase_rest_density"]], dtype=np.float64)
        # sph_config.py:165-185 (int fields truncate: wc_gamma, cs, iter bounds)
        p.divergence_threshold = rnd(cfg["solver_divergence_threshold"])
        p.compression_threshold = rnd(cfg["solver_compression_threshold"])
        p.iter_min = int(cfg["solver_iter_threshold_min"])
        p.iter_max = int(cfg["solver_iter_threshold_max"])
        p.cs = int(cfg["solver_cs"])
        p.wc_gamma = int(cfg["solver_wc_gamma"])
        p.cfl_factor = rnd(cfg["solver_cfl_factor"])
        p.fbm_diffusion = rnd(cfg["solver_fbm_diffusion_term"])
        p.fbm_convection = rnd(cfg["solver_fbm_convection_term"])
        p.surface_tension_gamma = rnd(cfg["solver_surface_tension_gamma"])
        # sph_config.py:196-202
        h = rnd(p.part_size * 2)
        p.h = h
        p.h2 = rnd(h ** 2)
        p.sig = {3: rnd(8 / math.pi / h ** 3), 2: rnd(40 / 7 / math.pi / h ** 2)}[p.dim]
        # sph_config.py:204-224 (ceil is taken on the field's precision)
        if taichi_f32:
            gs = np.ceil((p.rt.astype(F32) - p.lb.astype(F32)) / F32(h)).astype(np.float64)
        else:
            gs = np.ceil((p.rt - p.lb) / h)
        p.grid_size = gs.astype(np.int64)
        coder, node_num = [], 1
        for i in range(p.dim):
            coder.append(node_num)
            node_num *= int(p.grid_size[i])
        p.coder = np.array(coder, dtype=np.int64)
        p.node_num = node_num
        w = 2 * p.neighb_range + 1
        dice = [-p.neighb_range + i for i in range(w)]
        tmpl = np.zeros((w ** p.dim, p.dim), dtype=np.int64)
        for j in range(w ** p.dim):
            tmp = j
            for d in range(p.dim):
                digit = tmp // (w ** (p.dim - d - 1))
                tmp = tmp % (w ** (p.dim - d - 1))
                tmpl[j][p.dim - d - 1] = dice[digit]
        p.template = tmpl
        p.taichi_f32 = taichi_f32
        return p


# ----------------------------------------------------------------------------- kernels
def W(r, p):
    """Cubic spline, ``sph_util.py:16-25``."""
    q = r / p.h
    out = np.where(q <= 0.5, 6 * (q ** 3 - q ** 2) + 1, np.where(q < 1, 2 * (1 - q) ** 3, 0.0))
    return out * p.sig


def W_grad(r, p):
    """Radial derivative of W, ``sph_util.py:28-37``."""
    q = r / p.h
    out = np.where(q <= 0.5, 6 * (3 * q ** 2 - 2 * q), np.where(q < 1, -6 * (1 - q) ** 2, 0.0))
    return out * (p.sig / p.h)


def C(r, p):
    """Akinci cohesion spline, ``sph_util.py:4-13``."""
    q = r / p.h
    out = np.where(q <= 0.5, 2 * (1 - q) ** 3 * q ** 3 - 1 / 64,
                   np.where(q < 1, (1 - q) ** 3 * q ** 3, 0.0))
    return out * (32 / math.pi / p.h ** 3)


def node_encode(pos, p):
    """``int((pos - lb) // h)``, ``sph_util.py:65-67`` (float floordiv is floor(a/b))."""
    if p.taichi_f32:
        v = np.floor((pos.astype(F32) - p.lb.astype(F32)) / F32(p.h)).astype(np.float64)
    else:
        v = np.floor((pos - p.lb) / p.h)
    return np.trunc(v).astype(np.int64)


def dim_encode(struct, p):
    """``coder . cell``, ``sph_util.py:70-72``."""
    return struct @ p.coder


# ----------------------------------------------------------------------------- particle set
FIELDS_VEC = ("pos", "vel", "vel_adv", "acce", "acce_adv", "alpha_1", "normal", "pressure_force", "W_grad")
FIELDS_SCAL = ("mass", "rest_density", "rest_volume", "W", "sph_density", "sph_compression", "psi_adv",
               "alpha", "alpha_2", "fbm_zeta", "pressure")


class ParticleSet:
    """The per-particle arrays of ``Fluid`` (``sph_obj.py:24-86``), float64."""

    def __init__(self, n, p, uid):
        d, P = p.dim, p.phase_num
        self.n, self.uid = n, uid
        for f in FIELDS_VEC:
            setattr(self, f, np.zeros((n, d)))
        for f in FIELDS_SCAL:
            setattr(self, f, np.zeros(n))
        self.volume_frac = np.zeros((n, P))
        self.volume_frac_tmp = np.zeros((n, P))
        self.drift_vel = np.zeros((n, P, d))
        self.flag = np.zeros(n, dtype=np.int64)
        self.ones = np.ones(n)
        self.neighb_cell_seq = np.zeros(n, dtype=np.int64)
        self.neighb_cell_structured_seq = np.zeros((n, d), dtype=np.int64)
        self.compression = 0.0
        self.general_flag = 0
        self.statistics_kinetic_energy = 0.0
        self.statistics_gravity_potential_energy = 0.0
        # aliases, sph_obj.py:65-73
        if p.solver_type == "VFSPH":
            self._alias = ("rest_volume", "sph_compression", "ones")
        else:
            self._alias = ("mass", "sph_density", "rest_density")

    @property
    def X(self):
        return getattr(self, self._alias[0])

    @property
    def sph_psi(self):
        return getattr(self, self._alias[1])

    @property
    def rest_psi(self):
        return getattr(self, self._alias[2])

    @property
    def fbm_acce(self):
        return self.acce

    @fbm_acce.setter
    def fbm_acce(self, v):
        self.acce = v


class Pairs:
    """Candidate pairs of one (obj, nobj) sweep with their geometry."""

    def __init__(self, i, j, xij):
        self.i, self.j, self.xij = i, j, xij
        self.r = np.sqrt(np.einsum("ij,ij->i", xij, xij)) if len(i) else np.zeros(0)


class Grid:
    """Counting-sort cell grid of all particle sets, ``sph_obj.py:280-323``."""

    def __init__(self, p, sets):
        self.p = p
        self.members = {}
        for s in sets:
            struct = node_encode(s.pos, p)
            code = dim_encode(struct, p)
            s.neighb_cell_structured_seq = struct
            s.neighb_cell_seq = code
            valid = (code > 0) & (code < p.node_num)
            ids = np.nonzero(valid)[0]
            order = np.argsort(code[ids], kind="stable")
            self.members[s.uid] = (ids[order], code[ids][order])

    def pairs(self, obj, nobj):
        """Every (i, j) the reference's template loop visits (``sph.py:52-60``)."""
        i, j = self.candidates(obj.neighb_cell_structured_seq, nobj)
        return Pairs(i, j, obj.pos[i] - nobj.pos[j])

    def candidates(self, base, nobj):
        """(i, j): members j of nobj in the template cells around cell base[i]."""
        p = self.p
        ids, codes = self.members[nobj.uid]
        I, J = [], []
        n = len(base)
        for t in p.template:
            q = dim_encode(base + t, p)
            ok = (q > 0) & (q < p.node_num)
            lo = np.searchsorted(codes, q, "left")
            hi = np.searchsorted(codes, q, "right")
            cnt = np.where(ok, hi - lo, 0)
            tot = int(cnt.sum())
            if tot == 0:
                continue
            ii = np.repeat(np.arange(n), cnt)
            start = np.repeat(lo, cnt)
            off = np.arange(tot) - np.repeat(np.cumsum(cnt) - cnt, cnt)
            I.append(ii)
            J.append(ids[start + off])
        if I:
            return np.concatenate(I), np.concatenate(J)
        return np.zeros(0, dtype=np.int64), np.zeros(0, dtype=np.int64)


def _sum(idx, vals, n):
    if vals.ndim == 1:
        return np.bincount(idx, weights=vals, minlength=n)[:n] if n else np.zeros(0)
    out = np.zeros((n,) + vals.shape[1:])
    np.add.at(out, idx, vals)
    return out


# ----------------------------------------------------------------------------- sph.py kernels
def SPH_clean_value(obj):
    """``sph.py:22-38``."""
    obj.general_flag = 1
    for f in ("W", "sph_compression", "sph_density", "alpha_2"):
        getattr(obj, f)[:] = 0
    obj.flag[:] = 0
    for f in ("W_grad", "acce", "acce_adv", "alpha_1", "pressure_force"):
        getattr(obj, f)[:] = 0
    obj.drift_vel[:] = 0


def cfl_condition(fluid, p):
    """``sph.py:41-47`` (if_cfl is read but never consulted)."""
    dt = p.part_size / p.cs
    if fluid.n:
        vn = np.sqrt(np.einsum("ij,ij->i", fluid.vel, fluid.vel))
        m = vn > 1e-4
        if m.any():
            dt = min(dt, float(np.min(p.part_size / vn[m] * p.cfl_factor)))
    if p.taichi_f32:
        dt = float(F32(dt))
    return dt


def SPH_prepare_attr(pr, obj, nobj, p):
    """``sph.py:50-64`` (self term included: r = 0 gives W(0))."""
    Wr = W(pr.r, p)
    obj.W += _sum(pr.i, Wr, obj.n)
    obj.sph_compression += _sum(pr.i, Wr * nobj.rest_volume[pr.j], obj.n)
    obj.sph_density += _sum(pr.i, Wr * nobj.mass[pr.j], obj.n)


def _unit_grad(pr, p):
    m = pr.r > 0
    g = np.zeros_like(pr.xij)
    g[m] = pr.xij[m] / pr.r[m, None] * W_grad(pr.r[m], p)[:, None]
    return m, g


def SPH_prepare_alpha_1(pr, obj, nobj, p):
    """``sph.py:67-81``."""
    m, g = _unit_grad(pr, p)
    obj.alpha_1 += _sum(pr.i[m], nobj.X[pr.j[m], None] * g[m], obj.n)


def SPH_prepare_alpha_2(pr, obj, nobj, p):
    """``sph.py:84-97``."""
    m = pr.r > 0
    wg = W_grad(pr.r[m], p)
    j = pr.j[m]
    obj.alpha_2 += _sum(pr.i[m], wg ** 2 * nobj.X[j] ** 2 / nobj.mass[j], obj.n)


def SPH_prepare_alpha(obj):
    """``sph.py:100-105``."""
    obj.alpha[:] = np.einsum("ij,ij->i", obj.alpha_1, obj.alpha_1) / obj.mass + obj.alpha_2
    obj.alpha[:] = np.where(obj.alpha < 1e-4, 1e-4, obj.alpha)


def SPH_advection_gravity_acc(obj, p):
    """``sph.py:108-111``."""
    obj.acce_adv += p.gravity


def SPH_advection_viscosity_acc(pr, obj, nobj, p):
    """``sph.py:114-129`` with ``W_lap`` from ``sph_util.py:40-43``."""
    m = pr.r > 0
    i, j, x, r = pr.i[m], pr.j[m], pr.xij[m], pr.r[m]
    Vj = nobj.X[j] / nobj.sph_psi[j]
    A = obj.vel[i] - nobj.vel[j]
    lap = (2 * (2 + p.dim) * Vj * W_grad(r, p))[:, None] * (x / r[:, None]) * \
        (np.einsum("ij,ij->i", A, x) / (0.01 * p.h2 + r ** 2))[:, None]
    obj.acce_adv += _sum(i, lap * (p.viscosity / obj.rest_density[i])[:, None], obj.n)


def SPH_advection_surface_tension_acc(pr, obj, nobj, p):
    """``sph.py:132-166``: normals, then cohesion + curvature over all candidates."""
    m, g = _unit_grad(pr, p)
    i, j = pr.i[m], pr.j[m]
    obj.normal[:] = 0
    obj.normal += _sum(i, (-nobj.X[j] / nobj.sph_psi[j])[:, None] * g[m], obj.n)
    obj.normal *= p.h
    sel = m & (obj.volume_frac[pr.i, 0] > 0.99) & (nobj.volume_frac[pr.j, 0] > 0.99)
    i, j, x, r = pr.i[sel], pr.j[sel], pr.xij[sel], pr.r[sel]
    gam = p.surface_tension_gamma
    coh = (-gam * nobj.mass[j] * C(r, p))[:, None] * x / r[:, None]
    cur = gam * (obj.normal[i] - nobj.normal[j])
    fac = 2 * obj.rest_psi[i] / (obj.sph_psi[i] + nobj.sph_psi[j])
    obj.acce_adv += _sum(i, fac[:, None] * (coh + cur), obj.n)


def IPPE_adv_psi_init(obj):
    """``sph.py:196-199``."""
    obj.psi_adv[:] = obj.sph_psi - obj.rest_psi


def IPPE_adv_psi(pr, obj, nobj, p, dt):
    """``sph.py:202-216``."""
    m, g = _unit_grad(pr, p)
    i, j = pr.i[m], pr.j[m]
    dv = obj.vel_adv[i] - nobj.vel_adv[j]
    obj.psi_adv += _sum(i, np.einsum("ij,ij->i", g[m], dv) * nobj.X[j] * dt, obj.n)


def IPPE_psi_adv_non_negative(obj):
    """``sph.py:219-226``."""
    obj.psi_adv[:] = np.where(obj.psi_adv < 0, 0, obj.psi_adv)
    with np.errstate(invalid="ignore", divide="ignore"):
        obj.compression = float(np.sum(obj.psi_adv / obj.rest_psi)) / obj.n if obj.n else float("nan")


def IPPE_update_vel_adv(pr, obj, nobj, p, dt):
    """``sph.py:229-244`` (Jacobi: reads psi_adv and alpha, writes vel_adv of i)."""
    m, g = _unit_grad(pr, p)
    i, j = pr.i[m], pr.j[m]
    coef = obj.psi_adv[i] * nobj.X[j] / obj.alpha[i] + nobj.psi_adv[j] * obj.X[i] / nobj.alpha[j]
    obj.vel_adv += _sum(i, (-(1 / dt) * coef / obj.mass[i])[:, None] * g[m], obj.n)


def WC_pressure_val(obj, p):
    """``sph.py:169-176``: p = rho0 cs^2 / gamma ((rho / rho0)^7 - 1), clamped at 0."""
    pr = (obj.rest_density * p.cs ** 2 / p.wc_gamma) * ((obj.sph_density / obj.rest_density) ** 7 - 1)
    obj.pressure[:] = np.maximum(pr, 0.0)


def WC_pressure_acce(pr, obj, nobj, p):
    """``sph.py:179-193``: acce_adv -= (p_i / rho_i^2 + p_j / rho_j^2) m_j W'(r) x_ij / r."""
    m = pr.r > 0
    i, j, x, r = pr.i[m], pr.j[m], pr.xij[m], pr.r[m]
    pt = obj.pressure[i] / obj.sph_density[i] ** 2 + nobj.pressure[j] / nobj.sph_density[j] ** 2
    obj.acce_adv += _sum(i, (-pt * nobj.mass[j] * W_grad(r, p) / r)[:, None] * x, obj.n)


def map_velocity(grid, gpos, nobj, p):
    """``sph.py:382-397``: velocity at grid nodes gpos [G, dim] from the template
    cells of the cell grid built at the step's start and nobj's current state."""
    i, j = grid.candidates(node_encode(gpos, p), nobj)
    x = gpos[i] - nobj.pos[j]
    r = np.sqrt(np.einsum("ij,ij->i", x, x))
    w = nobj.X[j] / nobj.sph_psi[j] * W(r, p)
    return _sum(i, w[:, None] * nobj.vel[j], len(gpos))


def grid_positions(lb, dist, shape):
    """Node positions of ``Grid`` (``sph_obj.py:341-344``), C order."""
    idx = np.stack(np.meshgrid(*[np.arange(n) for n in shape], indexing="ij"), -1).reshape(-1, len(shape))
    return np.asarray(lb, dtype=np.float64) + idx * float(dist)


def SPH_advection_update_vel_adv(obj, dt):
    """``sph.py:247-250``."""
    obj.vel_adv[:] = obj.vel + obj.acce_adv * dt


def SPH_update_pos(obj, dt):
    """``sph.py:265-269``."""
    obj.vel[:] = obj.vel_adv
    obj.pos += obj.vel * dt


def SPH_update_energy(obj, p):
    """``sph.py:272-279``."""
    obj.statistics_kinetic_energy = float(np.sum(0.5 * obj.mass * np.einsum("ij,ij->i", obj.vel, obj.vel)))
    obj.statistics_gravity_potential_energy = float(
        np.sum(-obj.mass * p.gravity[1] * (obj.pos[:, 1] - p.lb[1])))


def SPH_update_mass(obj, p):
    """``sph.py:282-286``."""
    obj.rest_density[:] = obj.volume_frac @ p.phase_rest_density
    obj.mass[:] = obj.rest_density * obj.rest_volume


def SPH_FBM_clean_tmp(obj):
    """``sph.py:301-305``."""
    obj.volume_frac_tmp[:] = 0


def SPH_FBM_convect(pr, obj, nobj, p, dt):
    """``sph.py:329-363``: drift velocities, then the convective flux."""
    rho_k = p.phase_rest_density
    g = p.gravity
    with np.errstate(invalid="ignore", divide="ignore"):
        obj.acce_adv[:] = (obj.vel_adv - obj.vel) / dt
        obj.fbm_zeta[:] = np.sum(obj.volume_frac * (rho_k[None, :] - obj.rest_density[:, None]) / rho_k[None, :], axis=1)
        obj.fbm_acce = (obj.acce_adv - obj.fbm_zeta[:, None] * g) / (1 - obj.fbm_zeta[:, None])
        for k in range(p.phase_num):
            dv = (obj.volume_frac[:, k] * (rho_k[k] - obj.rest_density))[:, None] * (g - obj.fbm_acce)
            dw = obj.volume_frac[:, k] * rho_k[k]
            big = dw > 1e-6
            dv = np.where(big[:, None], dv / np.where(big, dw, 1.0)[:, None], dv * 0)
            dv = dv + (obj.fbm_acce - obj.acce_adv)
            obj.drift_vel[:, k, :] = dv * dt
    m, gr = _unit_grad(pr, p)
    m &= (obj.flag[pr.i] == 0) & (nobj.flag[pr.j] == 0)
    i, j, gg = pr.i[m], pr.j[m], gr[m]
    for k in range(p.phase_num):
        flux = obj.volume_frac[i, k, None] * obj.drift_vel[i, k] + nobj.volume_frac[j, k, None] * nobj.drift_vel[j, k]
        tmp = p.fbm_convection * dt * nobj.rest_volume[j] * np.einsum("ij,ij->i", flux, gg)
        obj.volume_frac_tmp[:, k] -= _sum(i, tmp, obj.n)


def SPH_FBM_diffuse(pr, obj, nobj, p, dt):
    """``sph.py:308-326``."""
    m = (pr.r > 0) & (obj.flag[pr.i] == 0) & (nobj.flag[pr.j] == 0)
    i, j, r = pr.i[m], pr.j[m], pr.r[m]
    w = dt * p.fbm_diffusion * nobj.rest_volume[j] * r * W_grad(r, p) / (r ** 2 + 0.01 * p.h2)
    obj.volume_frac_tmp += _sum(i, (obj.volume_frac[i] - nobj.volume_frac[j]) * w[:, None], obj.n)


def SPH_FBM_check_tmp(obj):
    """``sph.py:366-372``."""
    neg = np.any(obj.volume_frac + obj.volume_frac_tmp < 0, axis=1)
    obj.flag[neg] = 1
    obj.general_flag = int(neg.any())


def SPH_update_volume_frac(obj):
    """``sph.py:375-379``."""
    keep = ~(obj.flag > 0)
    obj.volume_frac[keep] += obj.volume_frac_tmp[keep]


# ----------------------------------------------------------------------------- step
class Stats:
    def __init__(self):
        self.dt = 0.0
        self.time_count = 0.0
        self.div_iter = 0
        self.incom_iter = 0
        self.fbm_passes = 0


def _solve(pff, pfb, fluid, bound, p, dt, tol):
    """One Jacobi solve loop, ``main.py:199-213`` / ``main.py:221-234``."""
    it = 0
    while it < p.iter_min or fluid.compression > tol:
        IPPE_adv_psi_init(fluid)
        IPPE_adv_psi(pff, fluid, fluid, p, dt)
        IPPE_adv_psi(pfb, fluid, bound, p, dt)
        IPPE_psi_adv_non_negative(fluid)
        IPPE_update_vel_adv(pff, fluid, fluid, p, dt)
        IPPE_update_vel_adv(pfb, fluid, bound, p, dt)
        it += 1
        if it > p.iter_max:
            break
    return it


def sph_step(fluid, bound, p, dt, fbm=False, max_fbm_passes=None, wc=False, map_grid=None):
    """``main.py:175-256`` (FBM block ``main.py:244-250`` when ``fbm``; the weakly
    compressible pressure block ``main.py:238-242`` when ``wc``; the particle-to-grid
    map ``main.py:254`` when ``map_grid`` = dict(lb, dist, shape), result in
    ``map_grid["vel"]``)."""
    grid = Grid(p, [fluid, bound])
    pff = grid.pairs(fluid, fluid)
    pfb = grid.pairs(fluid, bound)
    pbb = grid.pairs(bound, bound)
    pbf = grid.pairs(bound, fluid)
    SPH_clean_value(fluid)
    SPH_clean_value(bound)
    SPH_prepare_attr(pff, fluid, fluid, p)
    SPH_prepare_attr(pfb, fluid, bound, p)
    SPH_prepare_attr(pbb, bound, bound, p)
    SPH_prepare_attr(pbf, bound, fluid, p)
    SPH_prepare_alpha_1(pff, fluid, fluid, p)
    SPH_prepare_alpha_1(pfb, fluid, bound, p)
    SPH_prepare_alpha_2(pff, fluid, fluid, p)
    SPH_prepare_alpha_2(pbf, bound, fluid, p)
    SPH_prepare_alpha(fluid)
    SPH_prepare_alpha(bound)
    fluid.vel_adv[:] = fluid.vel
    k_div = _solve(pff, pfb, fluid, bound, p, dt, p.divergence_threshold)
    fluid.vel[:] = fluid.vel_adv
    SPH_advection_gravity_acc(fluid, p)
    SPH_advection_viscosity_acc(pff, fluid, fluid, p)
    SPH_advection_surface_tension_acc(pff, fluid, fluid, p)
    SPH_advection_update_vel_adv(fluid, dt)
    k_inc = _solve(pff, pfb, fluid, bound, p, dt, p.compression_threshold)
    if wc:
        WC_pressure_val(fluid, p)
        WC_pressure_acce(pff, fluid, fluid, p)
        WC_pressure_acce(pfb, fluid, bound, p)
        SPH_advection_update_vel_adv(fluid, dt)
    passes = 0
    if fbm:
        while fluid.general_flag > 0:
            SPH_FBM_clean_tmp(fluid)
            SPH_FBM_convect(pff, fluid, fluid, p, dt)
            SPH_FBM_diffuse(pff, fluid, fluid, p, dt)
            SPH_FBM_check_tmp(fluid)
            passes += 1
            if max_fbm_passes is not None and passes >= max_fbm_passes:
                break
        SPH_update_volume_frac(fluid)
    SPH_update_mass(fluid, p)
    SPH_update_pos(fluid, dt)
    SPH_update_energy(fluid, p)
    if map_grid is not None:
        gpos = grid_positions(map_grid["lb"], map_grid["dist"], map_grid["shape"])
        map_grid["vel"] = map_velocity(grid, gpos, fluid, p).reshape(tuple(map_grid["shape"]) + (p.dim,))
    return k_div, k_inc, passes


def run_substep(fluid, bound, p, stats, fbm=False, wc=False, map_grid=None):
    """One substep of ``run_step`` (``main.py:347-352``): CFL, clock, step."""
    dt = cfl_condition(fluid, p)
    stats.dt = dt
    stats.time_count += dt
    stats.div_iter, stats.incom_iter, stats.fbm_passes = sph_step(fluid, bound, p, dt, fbm=fbm, wc=wc,
                                                                  map_grid=map_grid)
    return stats


def sets_from_arrays(p, fluid_arrays, bound_arrays):
    """Build the two particle sets from dicts of per-particle arrays."""
    out = []
    for uid, arrs in enumerate((fluid_arrays, bound_arrays)):
        n = len(arrs["pos"])
        s = ParticleSet(n, p, uid)
        for k, v in arrs.items():
            setattr(s, k, np.array(v, dtype=getattr(s, k).dtype).reshape(getattr(s, k).shape))
        out.append(s)
    return out
