"""The solver: the reference's per-substep kernels behind one CUDA context.

``sph.py`` of Tichi_SPH exposes ~27 Taichi kernels that ``main.py:175-256``
(``sph_step``) calls in a fixed order.  Here that whole sequence is one call of
the C ABI (``tsph_sph_step`` / ``tsph_substep``), replayed as a CUDA graph with
device-side solver loops.  :class:`Solver` owns the context; the module-level
``cfl_condition`` / ``sph_step`` mirror the reference's entry points.

Kernel-level composition.  The module-level functions named after the
reference's kernels (``SPH_prepare_attr(ngrid, obj, nobj)``, ``IPPE_adv_psi``,
``IPPE_update_vel_adv``, ``SPH_advection_*``, ``SPH_FBM_*``, ``SPH_update_*``,
...) let a caller write ``sph_step`` as ``main.py:175-256`` does, with its own
Python solver loops reading ``fluid.compression[None]``.  The CUDA path fuses
the reference's kernels into a few sweeps, so the calls are gathered into the
groups those sweeps compute, and a group runs (one C call) when its last call
arrives:

=================================================  =======================  ==========================
reference calls (main.py order)                    C entry                  runs at
=================================================  =======================  ==========================
``ngrid.clear_node/encode/mem_shift/fill_node``,    ``tsph_grid_build``      the last of the eight
``SPH_clean_value`` (fluid, bound)
``SPH_prepare_attr`` x4, ``_alpha_1`` x2,           ``tsph_density_alpha``   the last of the ten
``_alpha_2`` x2, ``_alpha`` x2
``SPH_vel_2_vel_adv``                               (part of the gather)     --
``IPPE_adv_psi_init``, ``IPPE_adv_psi`` (f,f)(f,b), ``tsph_adv_psi``         the last of the four; sets
``IPPE_psi_adv_non_negative``                                                ``fluid.compression[None]``
``IPPE_update_vel_adv`` (f,f)(f,b)                  ``tsph_update_vel_adv``  the second
``SPH_vel_adv_2_vel``, gravity / viscosity /        ``tsph_nonpressure``     ``SPH_advection_update_
surface tension (each optional),                                             vel_adv``
``SPH_advection_update_vel_adv``
``WC_pressure_val``, ``WC_pressure_acce`` (f,f)     ``tsph_wc_pressure``     ``SPH_advection_update_
(f,b), ``SPH_advection_update_vel_adv``                                      vel_adv``
``SPH_FBM_clean_tmp/convect/diffuse/check_tmp``     ``tsph_fbm_pass``        the last of the four; sets
                                                                             ``fluid.general_flag[None]``
``SPH_update_volume_frac`` (with the volume-        ``tsph_update``          the last of the group;
fraction update), ``SPH_update_mass/pos/energy``                             refreshes the scalars
=================================================  =======================  ==========================

A Jacobi iteration belongs to the divergence solve before the non-pressure
group and to the density solve after it.  A group left incomplete when a call
of another group arrives raises :class:`~tichi_sph_gb300._native.TsphError`
naming what is missing: each fused sweep computes all of its group's pair terms
(e.g. a density sweep without the fluid-boundary pairs does not exist).
Between ``tsph_grid_build`` and ``tsph_update`` the step's state lives in the
context; the particle arrays hold the previous step's values until the update
group has run.  A step composed in ``main.py``'s order equals the fused
``sph_step`` bit for bit (the same kernels in the same order).
"""
import torch

from . import _native
from ._native import check


def _stream_handle(device):
    return torch.cuda.current_stream(device).cuda_stream


class Solver:
    """One solver context for a (fluid, boundary) pair of particle sets.

    ``fbm`` enables the volume-fraction update block that the reference ships
    commented out (``main.py:244-250``), ``wcsph`` its weakly compressible
    pressure block (``main.py:238-242``); ``use_graph=False`` runs the solver loops
    host-driven, reading the convergence value every iteration as the reference
    does (``main.py:201,222``)."""

    def __init__(self, config, fluid, bound, fbm=False, use_graph=True, fbm_max_passes=1000, wcsph=False,
                 ngrid=None):
        if fluid.device.type != "cuda" or bound.device.type != "cuda":
            raise RuntimeError("tichi_sph_gb300: particle sets must live on a CUDA device")
        self.config = config
        self.fluid = fluid
        self.bound = bound
        self.fbm = bool(fbm)
        self.device = fluid.device
        L = _native.lib()
        self._lib = L
        self.wcsph = bool(wcsph)
        params = config.to_params(fbm_enabled=self.fbm, fbm_max_passes=fbm_max_passes, wcsph_enabled=self.wcsph)
        ctx = _native.CtxP()
        with torch.cuda.device(self.device):
            check(L.tsph_create(_native.C.byref(params), fluid.max_part_num, bound.max_part_num,
                                _native.C.byref(ctx)), "tsph_create")
        self.ctx = ctx
        self.set_graph_mode(use_graph)
        self.tpp = 1
        self._stats = _native.Stats()
        self._warn = _native.StatusWarner()
        # kernel-level composition: the reference's kernels find the solver
        # through their particle sets and grid
        self.composer = _Composer(self)
        fluid._solver = self
        bound._solver = self
        if ngrid is not None:
            ngrid._solver = self

    def set_graph_mode(self, use_graph):
        check(self._lib.tsph_set_graph_mode(self.ctx, 1 if use_graph else 0), "tsph_set_graph_mode")

    def set_threads_per_particle(self, tpp):
        """Lanes per particle of the neighbour-list sweeps (1, 2, 4, 8)."""
        check(self._lib.tsph_set_threads_per_particle(self.ctx, int(tpp)), "tsph_set_threads_per_particle")
        self.tpp = int(tpp)

    def autotune(self, candidates=(1, 2, 4, 8), reps=5):
        """Times the neighbour-list sweeps (Jacobi pair + advection) for each
        threads-per-particle setting on the current state and keeps the fastest.
        Returns {tpp: ms per Jacobi iteration + advection}."""
        res = {}
        for t in candidates:
            self.set_threads_per_particle(t)
            ph = self.profile_phases(reps=reps)
            res[t] = ph["psi"] + ph["vel"] + ph["advect"]
        best = min(res, key=res.get)
        self.set_threads_per_particle(best)
        return res

    def close(self):
        if getattr(self, "ctx", None):
            self._lib.tsph_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _sets(self):
        return _native.C.byref(self.fluid.native_set()), _native.C.byref(self.bound.native_set())

    def cfl_condition(self):
        """``cfl_condition(fluid)``, sph.py:41-47 (dt stays on the device)."""
        with torch.cuda.device(self.device):
            check(self._lib.tsph_cfl_condition(self.ctx, _native.C.byref(self.fluid.native_set()),
                                               _native.C.c_void_p(_stream_handle(self.device))),
                  "tsph_cfl_condition")

    def sph_step(self):
        """``sph_step()``, main.py:175-256, with the current dt."""
        f, b = self._sets()
        with torch.cuda.device(self.device):
            check(self._lib.tsph_sph_step(self.ctx, f, b, _native.C.c_void_p(_stream_handle(self.device))),
                  "tsph_sph_step")

    def substep(self):
        """cfl_condition + clock + sph_step (main.py:348-350) as one graph launch."""
        f, b = self._sets()
        with torch.cuda.device(self.device):
            check(self._lib.tsph_substep(self.ctx, f, b, _native.C.c_void_p(_stream_handle(self.device))),
                  "tsph_substep")

    # ------------------------------------------------------ kernel-level calls
    def _stream(self):
        return _native.C.c_void_p(_stream_handle(self.device))

    def grid_build(self):
        """``tsph_grid_build``: starts a step (grid, clean values, gather)."""
        f, b = self._sets()
        with torch.cuda.device(self.device):
            check(self._lib.tsph_grid_build(self.ctx, f, b, self._stream()), "tsph_grid_build")

    def density_alpha(self):
        """``tsph_density_alpha``: SPH_prepare_attr / _alpha_1 / _alpha_2 / _alpha."""
        with torch.cuda.device(self.device):
            check(self._lib.tsph_density_alpha(self.ctx, self._stream()), "tsph_density_alpha")

    def adv_psi(self, kind, read=True):
        """``tsph_adv_psi``: one Jacobi sweep A; returns the compression if ``read``."""
        out = _native.C.c_double(0.0)
        ptr = _native.C.byref(out) if read else None
        with torch.cuda.device(self.device):
            check(self._lib.tsph_adv_psi(self.ctx, int(kind), ptr, self._stream()), "tsph_adv_psi")
        return float(out.value) if read else None

    def update_vel_adv(self, kind):
        """``tsph_update_vel_adv``: one Jacobi sweep B."""
        with torch.cuda.device(self.device):
            check(self._lib.tsph_update_vel_adv(self.ctx, int(kind), self._stream()), "tsph_update_vel_adv")

    def solve(self, kind, tol=-1.0, it_min=-1, it_max=-1):
        """``tsph_solve``: a whole solver loop; returns (iterations, compression)."""
        it = _native.C.c_int32(0)
        err = _native.C.c_double(0.0)
        with torch.cuda.device(self.device):
            check(self._lib.tsph_solve(self.ctx, int(kind), float(tol), int(it_min), int(it_max),
                                       _native.C.byref(it), _native.C.byref(err), self._stream()), "tsph_solve")
        return int(it.value), float(err.value)

    def nonpressure(self, terms=_native.TERM_ALL):
        """``tsph_nonpressure``: the non-pressure forces selected by ``terms``."""
        with torch.cuda.device(self.device):
            check(self._lib.tsph_nonpressure(self.ctx, int(terms), self._stream()), "tsph_nonpressure")

    def wc_pressure(self):
        """``tsph_wc_pressure``: the weakly compressible pressure block."""
        with torch.cuda.device(self.device):
            check(self._lib.tsph_wc_pressure(self.ctx, _native.C.byref(self.bound.native_set()), self._stream()),
                  "tsph_wc_pressure")

    def fbm_pass(self):
        """``tsph_fbm_pass``: one volume-fraction pass; returns general_flag."""
        gf = _native.C.c_int32(0)
        with torch.cuda.device(self.device):
            check(self._lib.tsph_fbm_pass(self.ctx, _native.C.byref(gf), self._stream()), "tsph_fbm_pass")
        return int(gf.value)

    def update(self):
        """``tsph_update``: ends the step and writes every field back."""
        f, b = self._sets()
        with torch.cuda.device(self.device):
            check(self._lib.tsph_update(self.ctx, f, b, self._stream()), "tsph_update")

    def set_state(self, time_count=0.0, dt=0.0, compression=0.0):
        with torch.cuda.device(self.device):
            check(self._lib.tsph_set_state(self.ctx, float(time_count), float(dt), float(compression),
                                           _native.C.c_void_p(_stream_handle(self.device))), "tsph_set_state")

    def stats(self):
        """Synchronises and returns the step's scalars; also refreshes the
        reference-visible scalars (``config.dt[None]``, ``fluid.compression[None]``,
        ``fluid.statistics_*_energy[None]``, ``fluid.general_flag[None]``)."""
        with torch.cuda.device(self.device):
            check(self._lib.tsph_read_stats(self.ctx, _native.C.byref(self._stats),
                                            _native.C.c_void_p(_stream_handle(self.device))), "tsph_read_stats")
        s = self._stats
        self._warn(s.status)
        self.config.dt[None] = s.dt
        self.fluid.compression[None] = s.compression
        self.fluid.statistics_kinetic_energy[None] = s.kinetic_energy
        self.fluid.statistics_gravity_potential_energy[None] = s.potential_energy
        self.fluid.general_flag[None] = s.general_flag
        return {k: getattr(s, k) for k, _ in _native.Stats._fields_}

    def profile_phases(self, reps=10):
        """Mean milliseconds per launch of each step phase (CUDA events on the
        current stream); see ``tsph_profile_phases``."""
        out = (_native.C.c_float * len(_native.PHASES))()
        f, b = self._sets()
        with torch.cuda.device(self.device):
            check(self._lib.tsph_profile_phases(self.ctx, f, b, int(reps), out,
                                                _native.C.c_void_p(_stream_handle(self.device))),
                  "tsph_profile_phases")
        return dict(zip(_native.PHASES, [float(v) for v in out]))

    def map_velocity(self, grid):
        """``map_velocity(ngrid, grid, fluid)``, sph.py:382-397: fills ``grid.vel``
        from the fluid's current state and the cell grid of the last step."""
        C = _native.C
        lb = (C.c_float * 3)(*[float(x) for x in grid.lb] + [0.0] * (3 - len(grid.lb)))
        shape = (C.c_int32 * 3)(*[int(x) for x in grid.shape] + [1] * (3 - len(grid.shape)))
        out = grid.vel
        with torch.cuda.device(self.device):
            check(self._lib.tsph_map_velocity(self.ctx, C.byref(self.fluid.native_set()), lb, float(grid.dist), shape,
                                              C.cast(out.data_ptr(), C.POINTER(C.c_float)),
                                              C.c_void_p(_stream_handle(self.device))), "tsph_map_velocity")

    def neighbor_stats(self):
        """Per-particle neighbour counts (fluid, boundary) and set hashes."""
        nf, nb = self.fluid.part_num[None], self.bound.part_num[None]
        dev = self.device
        fc = torch.zeros((max(nf, 1), 2), dtype=torch.int32, device=dev)
        bc = torch.zeros((max(nb, 1), 2), dtype=torch.int32, device=dev)
        fh = torch.zeros(max(nf, 1), dtype=torch.int64, device=dev)
        bh = torch.zeros(max(nb, 1), dtype=torch.int64, device=dev)
        f, b = self._sets()
        u64p = _native.C.POINTER(_native.C.c_uint64)
        with torch.cuda.device(dev):
            check(self._lib.tsph_neighbor_stats(
                self.ctx, f, b,
                _native.C.cast(fc.data_ptr(), _native._ip), _native.C.cast(fh.data_ptr(), u64p),
                _native.C.cast(bc.data_ptr(), _native._ip), _native.C.cast(bh.data_ptr(), u64p),
                _native.C.c_void_p(_stream_handle(dev))), "tsph_neighbor_stats")
        return fc[:nf], fh[:nf], bc[:nb], bh[:nb]

    def candidate_stats(self):
        """Per-particle number of candidates the density sweep's scan visits in
        the fluid and the boundary grid, as int32 tensors [n_f, 2] and [n_b, 2]."""
        nf, nb = self.fluid.part_num[None], self.bound.part_num[None]
        dev = self.device
        fc = torch.zeros((max(nf, 1), 2), dtype=torch.int32, device=dev)
        bc = torch.zeros((max(nb, 1), 2), dtype=torch.int32, device=dev)
        f, b = self._sets()
        with torch.cuda.device(dev):
            check(self._lib.tsph_candidate_stats(
                self.ctx, f, b, _native.C.cast(fc.data_ptr(), _native._ip), _native.C.cast(bc.data_ptr(), _native._ip),
                _native.C.c_void_p(_stream_handle(dev))), "tsph_candidate_stats")
        return fc[:nf], bc[:nb]


class _Composer:
    """Gathers the reference's kernel calls of a step into the groups the fused
    sweeps compute and runs each group's C entry when its last call arrives
    (the table in the module docstring)."""

    # (name, role) -> group; roles: "f" / "b" for (obj), "ff" / "fb" / "bb" / "bf" for (obj, nobj)
    GROUPS = {
        "grid": {("clear_node", ""), ("encode", "f"), ("encode", "b"), ("mem_shift", ""), ("fill_node", "f"),
                 ("fill_node", "b"), ("SPH_clean_value", "f"), ("SPH_clean_value", "b")},
        "density": {("SPH_prepare_attr", "ff"), ("SPH_prepare_attr", "fb"), ("SPH_prepare_attr", "bb"),
                    ("SPH_prepare_attr", "bf"), ("SPH_prepare_alpha_1", "ff"), ("SPH_prepare_alpha_1", "fb"),
                    ("SPH_prepare_alpha_2", "ff"), ("SPH_prepare_alpha_2", "bf"), ("SPH_prepare_alpha", "f"),
                    ("SPH_prepare_alpha", "b")},
        "vel_2_vel_adv": {("SPH_vel_2_vel_adv", "f")},
        "psi": {("IPPE_adv_psi_init", "f"), ("IPPE_adv_psi", "ff"), ("IPPE_adv_psi", "fb"),
                ("IPPE_psi_adv_non_negative", "f")},
        "vel": {("IPPE_update_vel_adv", "ff"), ("IPPE_update_vel_adv", "fb")},
        "advection": {("SPH_vel_adv_2_vel", "f"), ("SPH_advection_update_vel_adv", "f")},
        "wc": {("WC_pressure_val", "f"), ("WC_pressure_acce", "ff"), ("WC_pressure_acce", "fb"),
               ("SPH_advection_update_vel_adv", "f")},
        "fbm": {("SPH_FBM_clean_tmp", "f"), ("SPH_FBM_convect", "ff"), ("SPH_FBM_diffuse", "ff"),
                ("SPH_FBM_check_tmp", "f")},
        "update": {("SPH_update_mass", "f"), ("SPH_update_pos", "f"), ("SPH_update_energy", "f")},
    }
    # optional members: the non-pressure forces a caller may leave out
    OPTIONAL = {"advection": {("SPH_advection_gravity_acc", "f"): _native.TERM_GRAVITY,
                              ("SPH_advection_viscosity_acc", "ff"): _native.TERM_VISCOSITY,
                              ("SPH_advection_surface_tension_acc", "ff"): _native.TERM_SURFACE_TENSION},
                "update": {("SPH_update_volume_frac", "f"): 0}}

    def __init__(self, solver):
        self.solver = solver
        self.open = None      # group being gathered
        self.called = set()
        self.after_advection = False

    def role(self, *objs):
        r = ""
        for o in objs:
            if o is self.solver.fluid:
                r += "f"
            elif o is self.solver.bound:
                r += "b"
            else:
                raise _native.TsphError("this particle set does not belong to the solver the call reached")
        return r

    def _group_of(self, key):
        if self.open is not None and (key in self.GROUPS[self.open] or key in self.OPTIONAL.get(self.open, {})):
            return self.open
        if key == ("SPH_advection_update_vel_adv", "f"):
            return "advection"
        for g in ("grid", "density", "vel_2_vel_adv", "psi", "vel", "advection", "fbm", "update", "wc"):
            if key in self.GROUPS[g] or key in self.OPTIONAL.get(g, {}):
                return g
        raise _native.TsphError("%s%s is not a kernel of the composed step" % key)

    def call(self, name, role=""):
        key = (name, role)
        g = self._group_of(key)
        if self.open is not None and g != self.open:
            missing = sorted(self.GROUPS[self.open] - self.called)
            self.open, self.called = None, set()
            raise _native.TsphError(
                "composed sph_step: %s%s arrived while the %s group still lacks %s; the fused sweep of that "
                "group computes all of them" % (name, "(" + role + ")" if role else "", g,
                                               ", ".join("%s(%s)" % m for m in missing)))
        if key in self.called:
            self.open, self.called = None, set()
            raise _native.TsphError("composed sph_step: %s(%s) called twice in one group" % key)
        self.open = g
        self.called.add(key)
        if self.GROUPS[g] <= self.called:
            called, self.open, self.called = self.called, None, set()
            self._run(g, called)

    def _run(self, g, called):
        s = self.solver
        fl = s.fluid
        if g == "grid":
            s.grid_build()
            self.after_advection = False
            fl.general_flag[None] = 1  # SPH_clean_value (sph.py:24)
        elif g == "density":
            s.density_alpha()
        elif g == "psi":
            kind = _native.SOLVE_DENS if self.after_advection else _native.SOLVE_DIV
            fl.compression[None] = s.adv_psi(kind)
        elif g == "vel":
            s.update_vel_adv(_native.SOLVE_DENS if self.after_advection else _native.SOLVE_DIV)
        elif g == "advection":
            terms = 0
            for k, bit in self.OPTIONAL["advection"].items():
                if k in called:
                    terms |= bit
            s.nonpressure(terms)
            self.after_advection = True
        elif g == "wc":
            s.wc_pressure()
        elif g == "fbm":
            fl.general_flag[None] = s.fbm_pass()
        elif g == "update":
            if s.fbm and ("SPH_update_volume_frac", "f") not in called:
                raise _native.TsphError("composed sph_step: SPH_update_volume_frac(fluid) belongs to the update "
                                        "group when the volume-fraction update is on")
            s.update()
            s.stats()  # statistics_*_energy, dt and compression as the reference's fields hold them


def _composer(obj):
    sv = getattr(obj, "_solver", None)
    if sv is None:
        raise _native.TsphError("no solver is bound to this particle set (create a Solver for it first)")
    return sv.composer


def _pair(name, obj, nobj):
    c = _composer(obj)
    c.call(name, c.role(obj, nobj))


def _one(name, obj):
    c = _composer(obj)
    c.call(name, c.role(obj))


# The reference's kernels (sph.py), for composing sph_step as main.py:175-256 does.
def SPH_clean_value(obj):
    """sph.py:22-38."""
    _one("SPH_clean_value", obj)


def SPH_prepare_attr(ngrid, obj, nobj):
    """sph.py:50-64."""
    _pair("SPH_prepare_attr", obj, nobj)


def SPH_prepare_alpha_1(ngrid, obj, nobj):
    """sph.py:67-81."""
    _pair("SPH_prepare_alpha_1", obj, nobj)


def SPH_prepare_alpha_2(ngrid, obj, nobj):
    """sph.py:84-97."""
    _pair("SPH_prepare_alpha_2", obj, nobj)


def SPH_prepare_alpha(obj):
    """sph.py:100-105."""
    _one("SPH_prepare_alpha", obj)


def SPH_advection_gravity_acc(obj):
    """sph.py:108-111."""
    _one("SPH_advection_gravity_acc", obj)


def SPH_advection_viscosity_acc(ngrid, obj, nobj):
    """sph.py:114-129."""
    _pair("SPH_advection_viscosity_acc", obj, nobj)


def SPH_advection_surface_tension_acc(ngrid, obj, nobj):
    """sph.py:132-166."""
    _pair("SPH_advection_surface_tension_acc", obj, nobj)


def WC_pressure_val(obj):
    """sph.py:169-175."""
    _one("WC_pressure_val", obj)


def WC_pressure_acce(ngrid, obj, nobj):
    """sph.py:178-193."""
    _pair("WC_pressure_acce", obj, nobj)


def IPPE_adv_psi_init(obj):
    """sph.py:196-199."""
    _one("IPPE_adv_psi_init", obj)


def IPPE_adv_psi(ngrid, obj, nobj):
    """sph.py:202-216."""
    _pair("IPPE_adv_psi", obj, nobj)


def IPPE_psi_adv_non_negative(obj):
    """sph.py:219-226: also sets ``obj.compression[None]`` (a host read, as the
    reference's loop test makes it)."""
    _one("IPPE_psi_adv_non_negative", obj)


def IPPE_update_vel_adv(ngrid, obj, nobj):
    """sph.py:229-244."""
    _pair("IPPE_update_vel_adv", obj, nobj)


def SPH_vel_2_vel_adv(obj):
    """sph.py:253-256."""
    _one("SPH_vel_2_vel_adv", obj)


def SPH_vel_adv_2_vel(obj):
    """sph.py:259-262."""
    _one("SPH_vel_adv_2_vel", obj)


def SPH_advection_update_vel_adv(obj):
    """sph.py:247-250."""
    _one("SPH_advection_update_vel_adv", obj)


def SPH_update_pos(obj):
    """sph.py:265-269."""
    _one("SPH_update_pos", obj)


def SPH_update_energy(obj):
    """sph.py:272-279."""
    _one("SPH_update_energy", obj)


def SPH_update_mass(obj):
    """sph.py:282-286."""
    _one("SPH_update_mass", obj)


def SPH_FBM_clean_tmp(obj):
    """sph.py:301-305."""
    _one("SPH_FBM_clean_tmp", obj)


def SPH_FBM_convect(ngrid, obj, nobj):
    """sph.py:329-363."""
    _pair("SPH_FBM_convect", obj, nobj)


def SPH_FBM_diffuse(ngrid, obj, nobj):
    """sph.py:308-326."""
    _pair("SPH_FBM_diffuse", obj, nobj)


def SPH_FBM_check_tmp(obj):
    """sph.py:366-372."""
    _one("SPH_FBM_check_tmp", obj)


def SPH_update_volume_frac(obj):
    """sph.py:375-379."""
    _one("SPH_update_volume_frac", obj)


def fp32_fma_peak(device=None):
    """FP32 FMA rate of the GPU in TFLOP/s (independent FMA chains on every SM)."""
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    out = _native.C.c_double(0.0)
    with torch.cuda.device(dev):
        check(_native.lib().tsph_fp32_fma_peak(_native.C.byref(out), _native.C.c_void_p(_stream_handle(dev))),
              "tsph_fp32_fma_peak")
    return float(out.value)


def map_velocity(solver, grid):
    """Module-level form of ``map_velocity(ngrid, grid, fluid)`` (sph.py:382-397)."""
    solver.map_velocity(grid)


def cfl_condition(obj):
    """``cfl_condition(fluid)`` (sph.py:41-47): takes the fluid set (or its Solver)."""
    (obj if isinstance(obj, Solver) else _composer(obj).solver).cfl_condition()


def sph_step(solver):
    """Module-level form of ``sph_step()`` (main.py:175-256)."""
    solver.sph_step()
