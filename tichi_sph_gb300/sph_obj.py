"""Particle sets and bookkeeping objects: ``Fluid``, ``Ngrid``, ``GlobalVariable``.

Mirrors ``sph_obj.py`` of Tichi_SPH.  A :class:`Fluid` holds the reference's
per-particle fields (``sph_obj.py:24-63``) as contiguous PyTorch tensors of
capacity ``max_part_num`` on the GPU; the CUDA kernels read and write them in
place through the C ABI.  The emitters reproduce the reference's initial states
bit for bit (same numpy float32 / float64 arithmetic, ``sph_obj.py:102-180``).
"""
import numpy as np
import torch

from . import _native
from .sph_config import Scalar

F32 = np.float32

# Fields of the reference's Fluid, with their per-particle shape.
VEC_FIELDS = ["pos", "gui_2d_pos", "vel", "vel_adv", "acce", "acce_adv", "pressure_force", "W_grad",
              "alpha_1", "normal"]
SCALAR_FIELDS = ["mass", "rest_density", "rest_volume", "pressure", "W", "sph_compression", "sph_density",
                 "psi_adv", "alpha", "alpha_2", "fbm_zeta"]
INT_FIELDS = ["color", "flag", "neighb_cell_seq", "neighb_in_cell_seq"]


def _default_device():
    return torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu")


class Fluid:
    """One particle set (fluid or boundary), ``sph_obj.py:8-93``."""

    def __init__(self, max_part_num, config, uid, device=None):
        self.config = config
        self.max_part_num = int(max_part_num)
        self.uid = uid
        self.device = torch.device(device) if device is not None else _default_device()
        d = config.dim[None]
        P = config.phase_num[None]
        cap = self.max_part_num
        kw = dict(device=self.device)
        self.part_num = Scalar(0)
        for f in VEC_FIELDS:
            setattr(self, f, torch.zeros((cap, d), dtype=torch.float32, **kw))
        for f in SCALAR_FIELDS:
            setattr(self, f, torch.zeros(cap, dtype=torch.float32, **kw))
        for f in INT_FIELDS:
            setattr(self, f, torch.zeros(cap, dtype=torch.int32, **kw))
        self.color_vector = torch.zeros((cap, 3), dtype=torch.float32, **kw)
        self.volume_frac = torch.zeros((cap, P), dtype=torch.float32, **kw)
        self.volume_frac_tmp = torch.zeros((cap, P), dtype=torch.float32, **kw)
        self.drift_vel = torch.zeros((cap, P, d), dtype=torch.float32, **kw)
        self.neighb_cell_structured_seq = torch.zeros((cap, d), dtype=torch.int32, **kw)
        self.ones = torch.ones(cap, dtype=torch.int32, **kw)
        self.general_flag = Scalar(0)
        self.compression = Scalar(0.0)
        self.statistics_kinetic_energy = Scalar(0.0)
        self.statistics_gravity_potential_energy = Scalar(0.0)
        self._set = None
        self._set_key = None

    # aliases, sph_obj.py:65-73
    @property
    def X(self):
        return self.rest_volume if self.config.solver_type == "VFSPH" else self.mass

    @property
    def sph_psi(self):
        return self.sph_compression if self.config.solver_type == "VFSPH" else self.sph_density

    @property
    def rest_psi(self):
        return self.ones if self.config.solver_type == "VFSPH" else self.rest_density

    @property
    def fbm_acce(self):
        return self.acce

    # ---------------------------------------------------------------- emitters
    def scene_add_help_centering(self, start_pos, end_pos, spacing):
        """``sph_obj.py:102-107``."""
        end_pos = np.array(end_pos, dtype=np.float32)
        start_pos = np.array(start_pos, dtype=np.float32)
        matrix_shape = ((end_pos - start_pos + 1e-7) / spacing).astype(np.int32)
        padding = (end_pos - start_pos - matrix_shape * spacing) / 2
        return matrix_shape, padding

    def scene_add_cube(self, start_pos, end_pos, volume_frac, vel, color, relaxing_factor):
        """``sph_obj.py:110-114``."""
        spacing = float(self.config.part_size[1]) * relaxing_factor
        matrix_shape, padding = self.scene_add_help_centering(start_pos, end_pos, spacing)
        self.push_matrix(np.ones(matrix_shape, dtype=np.bool_), start_pos + padding, spacing, volume_frac, vel, color)

    def scene_add_from_inlet(self, center, size, norm, speed, volume_frac, color, relaxing_factor):
        """``sph_obj.py:117-137`` (3D only, as in the reference)."""
        spacing = float(self.config.part_size[1]) * relaxing_factor
        matrix_shape, padding = self.scene_add_help_centering([0] * len(size), size, spacing)
        seq = []
        if len(matrix_shape) == 2:
            if norm[0] == 0:
                u = np.array([1, 0, 0])
            else:
                u = _np_normalize(np.array([-norm[2] / norm[0], 0, 1]))
            v = _np_normalize(np.cross(u, norm))
            size = np.array(size) - padding
            start = np.array(center) - (size[0] * u + size[1] * v) / 2
            for i in range(matrix_shape[0]):
                for j in range(matrix_shape[1]):
                    seq.append(start + (float(i) * u + float(j) * v) * spacing)
        else:
            raise Exception("scenario ERROR: can only add 3D inlets.")
        pos_seq = np.array(seq)
        vel = np.array(norm) * speed
        self.push_part_seq(len(pos_seq), pos_seq, volume_frac, vel, color)

    def scene_add_box(self, start_pos, end_pos, layers, volume_frac, vel, color, relaxing_factor):
        """``sph_obj.py:140-151``."""
        spacing = float(self.config.part_size[1]) * relaxing_factor
        matrix_shape, padding = self.scene_add_help_centering(start_pos, end_pos, spacing)
        box = np.ones(matrix_shape, dtype=np.bool_)
        if len(matrix_shape) == 2:
            box[layers: matrix_shape[0] - layers, layers: matrix_shape[1] - layers] = False
        elif len(matrix_shape) == 3:
            box[layers: matrix_shape[0] - layers, layers: matrix_shape[1] - layers,
                layers: matrix_shape[2] - layers] = False
        else:
            raise Exception("scenario error: can only add 2D or 3D boxes")
        self.push_matrix(box, start_pos + padding, spacing, volume_frac, vel, color)

    def push_part_from_ply(self, p_sum, pos_seq, volume_frac, vel, color):
        """``sph_obj.py:153-154``."""
        self.push_part_seq(p_sum, pos_seq, volume_frac, vel, color)

    def push_matrix(self, matrix, start_position, spacing, volume_frac, vel, color):
        """``sph_obj.py:158-163``."""
        if len(matrix.shape) != self.config.dim[None]:
            raise Exception("scenario error: wrong object dimension")
        index = np.where(matrix == True)  # noqa: E712  (same expression as the reference)
        pos_seq = np.stack(index, axis=1) * spacing + start_position
        self.push_part_seq(len(pos_seq), pos_seq, volume_frac, vel, color)

    def push_part_seq(self, pushed_part_num, pos_seq, volume_frac, vel, color):
        """``sph_obj.py:165-180``: append particles, then recompute rest density
        and mass of every particle from its volume fractions.

        The reference writes past ``max_part_num`` unchecked; here it raises."""
        d = self.config.dim[None]
        cur = self.part_num[None]
        new = cur + int(pushed_part_num)
        if new > self.max_part_num:
            raise Exception("scenario error: %d particles exceed max_part_num %d of object %d"
                            % (new, self.max_part_num, self.uid))
        n = int(pushed_part_num)
        if n > 0:
            pos = np.asarray(pos_seq, dtype=np.float64).reshape(n, -1)[:, :d].astype(np.float32)
            dev = self.device
            self.pos[cur:new] = torch.from_numpy(pos).to(dev)
            self.volume_frac[cur:new] = torch.tensor(np.asarray(volume_frac, dtype=np.float32), device=dev)
            self.vel[cur:new] = torch.tensor(np.asarray(vel, dtype=np.float32)[:d], device=dev)
            self.rest_volume[cur:new] = float(self.config.part_size[d])
            self.color[cur:new] = int(color)
        self.part_num[None] = new
        self.update_mass_all()

    def update_mass_all(self):
        """rest_density = phase_rest_density . volume_frac; mass = rest_density * rest_volume
        over all particles (``sph_obj.py:178-180``, ``sph.py:282-286``)."""
        n = self.part_num[None]
        rho = torch.tensor(self.config.phase_rest_density[None], dtype=torch.float32, device=self.device)
        vf = self.volume_frac[:n]
        acc = torch.zeros(n, dtype=torch.float32, device=self.device)
        for k in range(vf.shape[1]):
            acc = acc + rho[k] * vf[:, k]
        self.rest_density[:n] = acc
        self.mass[:n] = acc * self.rest_volume[:n]

    # ---------------------------------------------------------------- C ABI view
    def native_set(self):
        """The ``tsph_set`` view of this object's tensors (rebuilt when part_num changes)."""
        key = (self.part_num[None],)
        if self._set is None or self._set_key != key:
            s = _native.Set()
            s.n = self.part_num[None]
            s.capacity = self.max_part_num
            for f in _native.SET_FLOAT_FIELDS:
                t = getattr(self, f)
                assert t.is_contiguous() and t.dtype == torch.float32
                setattr(s, f, _native.C.cast(t.data_ptr(), _native._fp))
            for f in _native.SET_INT_FIELDS:
                t = getattr(self, f)
                assert t.is_contiguous() and t.dtype == torch.int32
                setattr(s, f, _native.C.cast(t.data_ptr(), _native._ip))
            self._set = s
            self._set_key = key
        return self._set


def _np_normalize(v):
    """``sph_util.py:74-75``."""
    return v / np.linalg.norm(v)


class Ngrid:
    """The reference's neighbour grid, ``sph_obj.py:281-323``.

    The cell grids themselves live inside the solver's CUDA context (one sorted
    grid per particle set, built every step).  The methods below are the
    reference's calls as ``main.py:178-183`` makes them; with a solver bound
    (``Solver(..., ngrid=ngrid)``, which :class:`~tichi_sph_gb300.simulation.Simulation`
    does) they take part in a step composed from the reference's kernels, see
    :mod:`tichi_sph_gb300.sph`: the grid is built once all six calls and both
    ``SPH_clean_value`` calls of the step have been made."""

    def __init__(self, config):
        self.config = config
        self._solver = None

    def _composer(self):
        if self._solver is None:
            raise RuntimeError("Ngrid: no solver is bound to this grid (create the Solver with ngrid=...)")
        return self._solver.composer

    def clear_node(self):
        """``Ngrid.clear_node``, sph_obj.py:295-298."""
        self._composer().call("clear_node")

    def encode(self, obj):
        """``Ngrid.encode``, sph_obj.py:300-306."""
        c = self._composer()
        c.call("encode", c.role(obj))

    def mem_shift(self):
        """``Ngrid.mem_shift``, sph_obj.py:308-314."""
        self._composer().call("mem_shift")

    def fill_node(self, obj):
        """``Ngrid.fill_node``, sph_obj.py:316-323."""
        c = self._composer()
        c.call("fill_node", c.role(obj))


class Grid:
    """Eulerian grid of the particle-to-grid map, ``sph_obj.py:326-344``: node
    positions lb + I * dist with dist = part_size * neighb_grid_size ratio.
    The shape is ceil((rt - lb) / dist) per axis -- what ``sph_obj.py:326``
    means; its expression divides only ``lb`` (operator precedence).  ``vel``
    and ``pos`` are [*shape, dim] tensors (C order)."""

    def __init__(self, config, device=None):
        d = config.dim[None]
        self.dim = d
        self.lb = np.array([float(x) for x in config.sim_space_lb[None]], dtype=np.float32)
        rt = np.array([float(x) for x in config.sim_space_rt[None]], dtype=np.float32)
        self.dist = float(np.float32(float(config.part_size[1]) * float(config.neighb_grid_size_TO_global_part_size[None])))
        self.shape = tuple(int(x) for x in np.ceil((rt.astype(np.float64) - self.lb) / self.dist))
        self.size = int(np.prod(self.shape))
        self.device = torch.device(device) if device is not None else _default_device()
        idx = np.stack(np.meshgrid(*[np.arange(n) for n in self.shape], indexing="ij"), -1)
        self.pos = torch.as_tensor((self.lb + idx * np.float32(self.dist)).astype(np.float32), device=self.device)
        self.vel = torch.zeros(self.shape + (d,), dtype=torch.float32, device=self.device)


class GlobalVariable:
    """Host-side timers and counters, ``sph_obj.py:347-368`` (no window flags)."""

    def __init__(self):
        self.is_first_time = True
        self.time_real = 0
        self.time_start = 0
        self.time_count = float(0)
        self.time_counter = int(0)
        self.step_counter = int(0)
        self.frame_div_iter = 0
        self.frame_incom_iter = 0
        self.div_iter_count = 0
        self.incom_iter_count = 0
        self.show_window = False
        self.op_write_file = False
