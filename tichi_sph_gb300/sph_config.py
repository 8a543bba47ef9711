"""Configuration: the reference's config / scenario JSON schema and ``Config``.

Mirrors ``sph_config.py`` of Tichi_SPH (lines 13-235) without its import-time
side effects: :func:`load` (or :func:`from_argv` for the reference's ``-c`` /
``-s`` command line) builds a :class:`Config` whose attribute names and values
are those of the reference's ``Config`` singleton.  Every stored value is the
f32 (or i32) value a Taichi field with ``default_fp=f32`` would hold, since the
CUDA kernels compute with exactly those constants.

Scalars the reference reads as ``config.x[None]`` are :class:`Scalar` objects, so
the same expression works here; ``part_size``, ``kernel_h`` and ``kernel_sig``
are float32 arrays indexed like the reference's small fields.
"""
import getopt
import json
import math

import numpy as np

from . import _native

F32 = np.float32


def read_param(param, paramname):
    """``sph_config.py:13-16``."""
    if param is None:
        raise Exception("The parameter " + paramname + " is missing, or invalid parameter")
    return param


def read_array_param(param, default):
    """``sph_config.py:19-24``."""
    if param is None:
        return default
    elif len(param) != len(default):
        raise Exception("error: wrong array dimension in config file ", param)
    return param


class Scalar:
    """A 0-d field: ``s[None]`` reads / writes the value."""

    __slots__ = ("value",)

    def __init__(self, value=0):
        self.value = value

    def __getitem__(self, key):
        if key is not None:
            raise IndexError("0-d field: index with [None]")
        return self.value

    def __setitem__(self, key, value):
        if key is not None:
            raise IndexError("0-d field: index with [None]")
        self.value = value

    def __repr__(self):
        return "Scalar(%r)" % (self.value,)


def _f32(x):
    return float(F32(x))


def _vec32(v):
    return np.array(v, dtype=F32)


def parse_args(argv):
    """The reference's getopt parsing, ``sph_config.py:27-40``.

    Accepts ``--scenarioFile`` as documented (the reference's long option is
    misspelled ``--secnarioFile`` in its handler, so the long form never worked).
    """
    opts, _ = getopt.getopt(argv, "c:s:", ["configFile=", "scenarioFile="])
    config_file = scenario_file = ""
    for opt, arg in opts:
        if opt in ("-c", "--configFile"):
            config_file = arg
        elif opt in ("-s", "--scenarioFile", "--secnarioFile"):
            scenario_file = arg
    return config_file, scenario_file


class Config:
    """Solver constants, ``sph_config.py:83-235``."""

    def __init__(self, config_buffer, scenario_buffer):
        self.config_buffer = config_buffer
        self.scenario_buffer = scenario_buffer
        env = scenario_buffer["sim_env"]
        sim_dim = read_param(env["sim_dim"], "sim_dim")
        phase_num = read_param(env["phase_num"], "phase_num")
        self.solver_type = read_param(config_buffer.get("solver_type"), "solver_type")
        if self.solver_type not in ("DFSPH", "VFSPH"):
            raise Exception("solver_type must be DFSPH or VFSPH")
        neighb_range = read_param(config_buffer.get("solver_neighb_range"), "solver_neighb_range")
        self.arch = config_buffer.get("arch")  # accepted and ignored: the path always runs on the GPU
        if int(sim_dim) not in (2, 3):
            raise Exception("sim_dim must be 2 or 3")
        if not 1 <= int(phase_num) <= _native.MAX_PHASES:
            raise Exception("phase_num must be in [1, %d]" % _native.MAX_PHASES)

        # init_sim_env, sph_config.py:145-163
        self.dim = Scalar(int(sim_dim))
        self.part_size = np.zeros(5, dtype=F32)
        self.part_size[1] = _f32(read_param(env["global_part_size"], "global_part_size"))
        self.dynamic_viscosity = Scalar(_f32(read_param(env["global_dynamic_viscosity"], "global_dynamic_viscosity")))
        self.sim_space_lb = Scalar(_vec32(read_param(env["sim_space_lb"], "sim_space_lb")))
        self.sim_space_rt = Scalar(_vec32(read_param(env["sim_space_rt"], "sim_space_rt")))
        self.gravity = Scalar(_vec32(read_param(env["gravity"], "gravity")))
        self.phase_num = Scalar(int(phase_num))
        self.phase_rest_density = Scalar(_vec32(read_param(env["phase_rest_density"], "phase_rest_density")))
        self.fluid_max_part_num = Scalar(int(read_param(scenario_buffer["fluid"]["max_part_num"], "fluid_max_part_num")))
        self.bound_max_part_num = Scalar(int(read_param(scenario_buffer["bound"]["max_part_num"], "bound_max_part_num")))
        self.phase_rgb = np.zeros((int(phase_num), 3), dtype=F32)
        for i in range(int(phase_num)):
            hx = int(env["phase_color_hex"][i], 16)
            self.phase_rgb[i] = [((hx & 0xFF0000) >> 16) / 255.0, ((hx & 0x00FF00) >> 8) / 255.0, (hx & 0x0000FF) / 255.0]
        ps = float(self.part_size[1])
        self.part_size[2] = _f32(math.pow(ps, 2))
        self.part_size[3] = _f32(math.pow(ps, 3))
        self.part_size[4] = _f32(math.pow(ps, 4))
        for v, n in ((self.sim_space_lb[None], "sim_space_lb"), (self.sim_space_rt[None], "sim_space_rt"),
                     (self.gravity[None], "gravity")):
            if len(v) != int(sim_dim):
                raise Exception("scenario error: %s must have %d components" % (n, int(sim_dim)))
        if len(self.phase_rest_density[None]) != int(phase_num):
            raise Exception("scenario error: phase_rest_density must have phase_num entries")

        # init_solver, sph_config.py:165-185 (int fields truncate)
        cb = config_buffer
        self.dt = Scalar(0.0)
        self.wc_gamma = Scalar(int(read_param(cb.get("solver_wc_gamma"), "solver_wc_gamma")))
        self.divergence_threshold = Scalar(_f32(read_param(cb.get("solver_divergence_threshold"), "solver_divergence_threshold")))
        self.compression_threshold = Scalar(_f32(read_param(cb.get("solver_compression_threshold"), "solver_compression_threshold")))
        self.iter_threshold_min = Scalar(int(read_param(cb.get("solver_iter_threshold_min"), "solver_iter_threshold_min")))
        self.iter_threshold_max = Scalar(int(read_param(cb.get("solver_iter_threshold_max"), "solver_iter_threshold_max")))
        self.if_cfl = Scalar(int(read_param(cb.get("solver_if_cfl"), "solver_if_cfl")))
        self.cs = Scalar(int(read_param(cb.get("solver_cs"), "solver_cs")))
        self.cfl_factor = Scalar(_f32(read_param(cb.get("solver_cfl_factor"), "solver_cfl_factor")))
        self.neighb_range = Scalar(int(read_param(cb.get("solver_neighb_range"), "solver_neighb_range")))
        self.neighb_grid_size_TO_global_part_size = Scalar(int(read_param(
            cb.get("solver_neighb_grid_size_TO_global_part_size"), "solver_neighb_grid_size_TO_global_part_size")))
        self.fbm_diffusion_term = Scalar(_f32(read_param(cb.get("solver_fbm_diffusion_term"), "solver_fbm_diffusion_term")))
        self.fbm_convection_term = Scalar(_f32(read_param(cb.get("solver_fbm_convection_term"), "solver_fbm_convection_term")))
        self.surface_tension_gamma = Scalar(_f32(read_param(cb.get("solver_surface_tension_gamma"), "solver_surface_tension_gamma")))
        if self.cs[None] == 0:
            raise Exception("solver_cs must be nonzero")

        # init_gui, sph_config.py:187-194 (values kept; there is no window here)
        self.gui_res = Scalar(cb.get("gui_res"))
        self.gui_part_zoomer = Scalar(cb.get("gui_part_zoomer"))
        self.gui_fps = Scalar(int(read_param(cb.get("gui_fps"), "gui_fps")))
        self.gui_canvas_bgcolor = Scalar(cb.get("gui_canvas_bgcolor"))
        self.gui_camera_pos = Scalar(cb.get("gui_camera_pos"))
        self.gui_camera_lookat = Scalar(cb.get("gui_camera_lookat"))

        # calculate_kernel_param, sph_config.py:196-202
        self.kernel_h = np.zeros(5, dtype=F32)
        self.kernel_sig = np.zeros(4, dtype=F32)
        self.kernel_h[1] = _f32(ps * 2)
        h = float(self.kernel_h[1])
        self.kernel_h[2] = _f32(math.pow(h, 2))
        self.kernel_h[3] = _f32(math.pow(h, 3))
        self.kernel_h[4] = _f32(math.pow(h, 4))
        self.kernel_sig[3] = _f32(8 / math.pi / h ** 3)
        self.kernel_sig[2] = _f32(40 / 7 / math.pi / h ** 2)

        # init_neighb_param + calculate_neighb_param, sph_config.py:204-224 (f32 ceil)
        rt, lb = self.sim_space_rt[None], self.sim_space_lb[None]
        self.neighb_grid_size = Scalar(np.ceil((rt - lb) / F32(h)).astype(F32))
        coder = np.ones(int(sim_dim), dtype=np.int64)
        node_num = 1
        for i in range(int(sim_dim)):
            coder[i] = node_num
            node_num *= int(self.neighb_grid_size[None][i])
        if node_num < 1:
            raise Exception("scenario error: sim_space_rt must exceed sim_space_lb on every axis")
        self.neighb_grid_coder = Scalar(coder)
        self.node_num = Scalar(node_num)
        w = 2 * int(neighb_range) + 1
        self.private_neighb_dice = np.array([-int(neighb_range) + i for i in range(w)], dtype=np.int64)
        tmpl = np.zeros((w ** int(sim_dim), int(sim_dim)), dtype=np.int64)
        for j in range(w ** int(sim_dim)):
            tmp = j
            for d in range(int(sim_dim)):
                digit = tmp // (w ** (int(sim_dim) - d - 1))
                tmp = tmp % (w ** (int(sim_dim) - d - 1))
                tmpl[j][int(sim_dim) - d - 1] = self.private_neighb_dice[digit]
        self.neighb_search_template = tmpl

    # -------------------------------------------------------------------- C ABI
    def to_params(self, fbm_enabled=False, fbm_max_passes=1000, wcsph_enabled=False):
        """The :class:`_native.Params` struct handed to ``tsph_create``."""
        p = _native.Params()
        d = self.dim[None]
        p.dim = d
        p.phase_num = self.phase_num[None]
        p.solver_type = _native.VFSPH if self.solver_type == "VFSPH" else _native.DFSPH
        p.neighb_range = self.neighb_range[None]
        p.part_size = float(self.part_size[1])
        p.kernel_h = float(self.kernel_h[1])
        p.kernel_h2 = float(self.kernel_h[2])
        p.kernel_sig = float(self.kernel_sig[d])
        gs = self.neighb_grid_size[None]
        for i in range(3):
            p.lb[i] = float(self.sim_space_lb[None][i]) if i < d else 0.0
            p.gravity[i] = float(self.gravity[None][i]) if i < d else 0.0
            p.grid_size[i] = int(gs[i]) if i < d else 1
        p.node_num = int(self.node_num[None])
        p.viscosity = float(self.dynamic_viscosity[None])
        for i, v in enumerate(self.phase_rest_density[None]):
            p.phase_rest_density[i] = float(v)
        p.divergence_threshold = float(self.divergence_threshold[None])
        p.compression_threshold = float(self.compression_threshold[None])
        p.iter_min = self.iter_threshold_min[None]
        p.iter_max = self.iter_threshold_max[None]
        p.cs = self.cs[None]
        p.cfl_factor = float(self.cfl_factor[None])
        p.fbm_diffusion = float(self.fbm_diffusion_term[None])
        p.fbm_convection = float(self.fbm_convection_term[None])
        p.surface_tension_gamma = float(self.surface_tension_gamma[None])
        p.fbm_enabled = 1 if fbm_enabled else 0
        p.fbm_max_passes = int(fbm_max_passes)
        p.wc_gamma = int(self.wc_gamma[None])
        p.wcsph_enabled = 1 if wcsph_enabled else 0
        return p


def load(config_file, scenario_file):
    """Reads the two JSON files (``sph_config.py:45-57``) and builds a Config."""
    with open(config_file) as f:
        config_buffer = json.load(f)
    with open(scenario_file) as f:
        scenario_buffer = json.load(f)
    return Config(config_buffer, scenario_buffer)


def from_argv(argv):
    """``main.py -c <config> -s <scenario>`` semantics."""
    c, s = parse_args(argv)
    return load(c, s)
