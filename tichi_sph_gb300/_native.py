"""ctypes binding of ``include/tichi_sph.h`` (the C ABI of the CUDA hot path).

The library is loaded from ``tichi_sph_gb300/_lib/libtichi_sph.so`` (built by
``tichi_sph_gb300.build.build()``).  There is no fallback: if the library is
missing, :func:`lib` raises, so nothing silently runs anywhere but the GPU.
"""
import ctypes as C
import os
import warnings

from . import build as _build

MAX_PHASES = 8

OK, ERR_INVALID, ERR_CAPACITY, ERR_CUDA, ERR_STATE = 0, 1, 2, 3, 4
ST_NONFINITE_POS, ST_DIV_ITER_CAP, ST_DENS_ITER_CAP, ST_FBM_PASS_CAP, ST_OUTSIDE_GRID = 1, 2, 4, 8, 16
DFSPH, VFSPH = 0, 1
SOLVE_DIV, SOLVE_DENS = 0, 1
TERM_GRAVITY, TERM_VISCOSITY, TERM_SURFACE_TENSION, TERM_ALL = 1, 2, 4, 7

_STATUS_TEXT = (
    (ST_NONFINITE_POS, "a fluid or boundary position is not finite (the particle has no cell and no neighbours)"),
    (ST_OUTSIDE_GRID, "particles lie outside the neighbour grid (sim_space_lb .. sim_space_rt) and have no "
                      "neighbours"),
    (ST_DIV_ITER_CAP, "the divergence-free solve stopped at solver_iter_threshold_max"),
    (ST_DENS_ITER_CAP, "the constant-density solve stopped at solver_iter_threshold_max"),
    (ST_FBM_PASS_CAP, "the volume-fraction pass loop stopped at its pass cap"),
)


def status_messages(status):
    """The conditions a step's status bits (``TSPH_ST_*``) report, in words."""
    return [text for bit, text in _STATUS_TEXT if status & bit]


class StatusWarner:
    """Reports a step's status bits as RuntimeWarnings, each condition once per
    solver (and scene).  The reference goes on silently in all of these cases
    (cells out of range are skipped, sph.py:52-60; the solver loops break at
    their cap, main.py:213, 233), and so does the step; the warning only tells."""

    def __init__(self, scene=None):
        self.scene = scene
        self.seen = 0

    def __call__(self, status):
        new = int(status) & ~self.seen
        if not new:
            return
        self.seen |= new
        where = "" if self.scene is None else " (scene %d)" % self.scene
        for text in status_messages(new):
            warnings.warn("tichi_sph_gb300: " + text + where, RuntimeWarning, stacklevel=3)

_f = C.c_float
_i32 = C.c_int32
_i64 = C.c_int64
_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int32)


class Params(C.Structure):
    _fields_ = [
        ("dim", _i32), ("phase_num", _i32), ("solver_type", _i32), ("neighb_range", _i32),
        ("part_size", _f), ("kernel_h", _f), ("kernel_h2", _f), ("kernel_sig", _f),
        ("lb", _f * 3), ("grid_size", _i32 * 3), ("node_num", _i64),
        ("gravity", _f * 3), ("viscosity", _f),
        ("phase_rest_density", _f * MAX_PHASES),
        ("divergence_threshold", _f), ("compression_threshold", _f),
        ("iter_min", _i32), ("iter_max", _i32), ("cs", _i32), ("cfl_factor", _f),
        ("fbm_diffusion", _f), ("fbm_convection", _f), ("surface_tension_gamma", _f),
        ("fbm_enabled", _i32), ("fbm_max_passes", _i32), ("wc_gamma", _i32), ("wcsph_enabled", _i32),
    ]


SET_FLOAT_FIELDS = ["pos", "vel", "vel_adv", "acce", "acce_adv", "mass", "rest_density", "rest_volume",
                    "volume_frac", "volume_frac_tmp", "W", "sph_density", "sph_compression", "psi_adv",
                    "alpha", "alpha_1", "alpha_2", "normal", "drift_vel", "fbm_zeta", "pressure"]
SET_INT_FIELDS = ["flag", "neighb_cell_seq", "neighb_in_cell_seq", "neighb_cell_structured_seq"]


class Set(C.Structure):
    _fields_ = ([("n", _i64), ("capacity", _i64)] + [(f, _fp) for f in SET_FLOAT_FIELDS]
                + [(f, _ip) for f in SET_INT_FIELDS])


class Stats(C.Structure):
    _fields_ = [
        ("dt", C.c_double), ("time_count", C.c_double), ("compression", C.c_double),
        ("kinetic_energy", C.c_double), ("potential_energy", C.c_double),
        ("div_iter", _i32), ("incom_iter", _i32), ("fbm_passes", _i32), ("general_flag", _i32),
        ("status", _i32), ("fluid_in_grid", _i32), ("bound_in_grid", _i32), ("steps", _i32),
        ("total_div_iter", _i64), ("total_incom_iter", _i64), ("total_fbm_passes", _i64),
        ("max_dens_compression", C.c_double),
        ("launches_per_step", _i32), ("launches_per_iter", _i32), ("launches_per_pass", _i32), ("pad", _i32),
    ]


PHASES = ["cfl", "grid", "density", "psi", "vel", "advect", "unsort"]


class Ctx(C.Structure):
    pass


CtxP = C.POINTER(Ctx)

# name -> (restype, argtypes); the full list of symbols include/tichi_sph.h declares
SIGNATURES = {
    "tsph_create": (C.c_int, [C.POINTER(Params), _i64, _i64, C.POINTER(CtxP)]),
    "tsph_create_batch": (C.c_int, [C.POINTER(Params), C.c_int, C.POINTER(_i64), C.POINTER(_i64), C.POINTER(CtxP)]),
    "tsph_destroy": (C.c_int, [CtxP]),
    "tsph_set_graph_mode": (C.c_int, [CtxP, C.c_int]),
    "tsph_set_threads_per_particle": (C.c_int, [CtxP, C.c_int]),
    "tsph_cfl_condition": (C.c_int, [CtxP, C.POINTER(Set), C.c_void_p]),
    "tsph_sph_step": (C.c_int, [CtxP, C.POINTER(Set), C.POINTER(Set), C.c_void_p]),
    "tsph_substep": (C.c_int, [CtxP, C.POINTER(Set), C.POINTER(Set), C.c_void_p]),
    "tsph_read_stats": (C.c_int, [CtxP, C.POINTER(Stats), C.c_void_p]),
    "tsph_read_scene_stats": (C.c_int, [CtxP, C.c_int, C.c_int, C.POINTER(Stats), C.c_void_p]),
    "tsph_set_state": (C.c_int, [CtxP, C.c_double, C.c_float, C.c_double, C.c_void_p]),
    "tsph_neighbor_stats": (C.c_int, [CtxP, C.POINTER(Set), C.POINTER(Set), _ip, C.POINTER(C.c_uint64),
                                      _ip, C.POINTER(C.c_uint64), C.c_void_p]),
    "tsph_candidate_stats": (C.c_int, [CtxP, C.POINTER(Set), C.POINTER(Set), _ip, _ip, C.c_void_p]),
    "tsph_fp32_fma_peak": (C.c_int, [C.POINTER(C.c_double), C.c_void_p]),
    "tsph_profile_phases": (C.c_int, [CtxP, C.POINTER(Set), C.POINTER(Set), C.c_int, _fp, C.c_void_p]),
    "tsph_fluid_density_noalloc": (C.c_int, [C.POINTER(Params), _fp, _fp, _fp, _i64, _fp, _fp, _fp, _i64,
                                             _fp, _fp, _fp, C.c_void_p]),
    "tsph_map_velocity": (C.c_int, [CtxP, C.POINTER(Set), _fp, C.c_float, _ip, _fp, C.c_void_p]),
    "tsph_tape_create": (C.c_int, [CtxP, C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "tsph_tape_destroy": (C.c_int, [C.c_void_p]),
    "tsph_substep_record": (C.c_int, [CtxP, C.POINTER(Set), C.POINTER(Set), C.c_void_p, C.c_int, C.c_void_p]),
    "tsph_density_record": (C.c_int, [CtxP, C.POINTER(Set), C.POINTER(Set), C.c_void_p, C.c_int, _fp,
                                      C.c_void_p]),
    "tsph_substep_adjoint": (C.c_int, [CtxP, C.c_void_p, C.c_int, _fp, _fp, _fp, _fp,
                                       C.POINTER(C.c_double), C.c_void_p]),
    "tsph_density_adjoint": (C.c_int, [CtxP, C.c_void_p, C.c_int, _fp, _fp, C.c_void_p]),
    "tsph_set_viscosity": (C.c_int, [CtxP, C.c_int, C.c_float]),
    "tsph_grid_build": (C.c_int, [CtxP, C.POINTER(Set), C.POINTER(Set), C.c_void_p]),
    "tsph_density_alpha": (C.c_int, [CtxP, C.c_void_p]),
    "tsph_adv_psi": (C.c_int, [CtxP, C.c_int, C.POINTER(C.c_double), C.c_void_p]),
    "tsph_update_vel_adv": (C.c_int, [CtxP, C.c_int, C.c_void_p]),
    "tsph_solve": (C.c_int, [CtxP, C.c_int, C.c_double, _i32, _i32, C.POINTER(_i32), C.POINTER(C.c_double),
                             C.c_void_p]),
    "tsph_nonpressure": (C.c_int, [CtxP, _i32, C.c_void_p]),
    "tsph_wc_pressure": (C.c_int, [CtxP, C.POINTER(Set), C.c_void_p]),
    "tsph_fbm_pass": (C.c_int, [CtxP, C.POINTER(_i32), C.c_void_p]),
    "tsph_update": (C.c_int, [CtxP, C.POINTER(Set), C.POINTER(Set), C.c_void_p]),
    "tsph_version": (C.c_char_p, []),
    "tsph_last_error": (C.c_char_p, []),
}

_LIB = None


def lib_path():
    return _build.LIB


def lib():
    """Loads the shared library (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        path = lib_path()
        if not os.path.exists(path):
            raise ImportError("tichi_sph_gb300: CUDA library %s is missing; run "
                              "`python -c 'import __graft_entry__ as g; g.build()'`" % path)
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


class TsphError(RuntimeError):
    pass


def check(rc, what):
    if rc != OK:
        msg = lib().tsph_last_error().decode(errors="replace")
        raise TsphError("%s failed (code %d): %s" % (what, rc, msg))
