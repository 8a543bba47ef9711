"""The solver: the reference's per-substep kernels behind one CUDA context.

``sph.py`` of Tichi_SPH exposes ~27 Taichi kernels that ``main.py:175-256``
(``sph_step``) calls in a fixed order.  Here that whole sequence is one call of
the C ABI (``tsph_sph_step`` / ``tsph_substep``), replayed as a CUDA graph with
device-side solver loops.  :class:`Solver` owns the context; the module-level
``cfl_condition`` / ``sph_step`` mirror the reference's entry points.
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

    def __init__(self, config, fluid, bound, fbm=False, use_graph=True, fbm_max_passes=1000, wcsph=False):
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


def cfl_condition(solver):
    """Module-level form of ``cfl_condition(fluid)`` (sph.py:41-47)."""
    solver.cfl_condition()


def sph_step(solver):
    """Module-level form of ``sph_step()`` (main.py:175-256)."""
    solver.sph_step()
