"""Batched form: many independent scenes stepped in the same launches.

The reference runs one scene per process (``main.py:8-12``).  ``BatchSolver``
steps S scenes of uneven sizes together: every scene keeps its own constants
(box, grid, rest density, thresholds), its own CFL time step, solver loops and
iteration counts, exactly as if it ran alone (``tsph_create_batch``).  The
scenes' particles live in one pair of concatenated particle sets; after
:func:`gather_scenes` each scene's ``Fluid`` objects are views into them, so the
reference-shaped per-scene API keeps working.
"""
import ctypes as C

import torch

from . import _native
from ._native import check
from .sph_obj import Fluid, VEC_FIELDS, SCALAR_FIELDS, INT_FIELDS


def _stream(device):
    return C.c_void_p(torch.cuda.current_stream(device).cuda_stream)


FIELDS = VEC_FIELDS + SCALAR_FIELDS + INT_FIELDS + ["volume_frac", "volume_frac_tmp", "drift_vel",
                                                   "neighb_cell_structured_seq", "ones", "color_vector"]


def gather_scenes(sims, device="cuda"):
    """Concatenates the fluid and boundary sets of initialised ``Simulation``s
    (scene order) into two device ``Fluid``s and rebinds every scene's fields to
    views of them.  Returns (fluid, bound, fluid_counts, bound_counts)."""
    cfg0 = sims[0].config
    nf = [s.fluid.part_num[None] for s in sims]
    nb = [s.bound.part_num[None] for s in sims]
    fluid = Fluid(max(sum(nf), 1), cfg0, 0, device=device)
    bound = Fluid(max(sum(nb), 1), cfg0, 1, device=device)
    for big, key, counts in ((fluid, "fluid", nf), (bound, "bound", nb)):
        off = 0
        for s, n in zip(sims, counts):
            obj = getattr(s, key)
            for f in FIELDS:
                src = getattr(obj, f)[:n]
                dst = getattr(big, f)
                dst[off:off + n] = src.to(device)
                setattr(obj, f, dst[off:off + n])
            obj.max_part_num = n
            obj.device = torch.device(device)
            obj._set = None
            off += n
        big.part_num[None] = off
    return fluid, bound, nf, nb


class BatchSolver:
    """One context stepping every scene of a batch (``tsph_create_batch``)."""

    def __init__(self, configs, fluid, bound, fluid_counts, bound_counts, fbm=False, use_graph=True,
                 fbm_max_passes=1000):
        if fluid.device.type != "cuda":
            raise RuntimeError("tichi_sph_gb300: particle sets must live on a CUDA device")
        S = len(configs)
        if len(fluid_counts) != S or len(bound_counts) != S:
            raise ValueError("one fluid and one boundary count per scene")
        self.configs = configs
        self.fluid, self.bound = fluid, bound
        self.device = fluid.device
        self.n_scenes = S
        L = _native.lib()
        self._lib = L
        params = (_native.Params * S)(*[c.to_params(fbm_enabled=fbm, fbm_max_passes=fbm_max_passes) for c in configs])
        fc = (C.c_int64 * S)(*fluid_counts)
        bc = (C.c_int64 * S)(*bound_counts)
        ctx = _native.CtxP()
        with torch.cuda.device(self.device):
            check(L.tsph_create_batch(params, S, fc, bc, C.byref(ctx)), "tsph_create_batch")
        self.ctx = ctx
        check(L.tsph_set_graph_mode(ctx, 1 if use_graph else 0), "tsph_set_graph_mode")
        self._stats = (_native.Stats * S)()

    def set_threads_per_particle(self, tpp):
        check(self._lib.tsph_set_threads_per_particle(self.ctx, int(tpp)), "tsph_set_threads_per_particle")

    def substep(self):
        """One substep of every scene (cfl_condition + clock + sph_step each)."""
        f, b = C.byref(self.fluid.native_set()), C.byref(self.bound.native_set())
        with torch.cuda.device(self.device):
            check(self._lib.tsph_substep(self.ctx, f, b, _stream(self.device)), "tsph_substep")

    def stats(self):
        """Per-scene scalars of the last substep (synchronises)."""
        with torch.cuda.device(self.device):
            check(self._lib.tsph_read_scene_stats(self.ctx, 0, self.n_scenes, self._stats, _stream(self.device)),
                  "tsph_read_scene_stats")
        if getattr(self, "_warn", None) is None:
            self._warn = [_native.StatusWarner(scene=i) for i in range(self.n_scenes)]
        for w, s in zip(self._warn, self._stats):
            w(s.status)
        return [{k: getattr(s, k) for k, _ in _native.Stats._fields_} for s in self._stats]

    def close(self):
        if getattr(self, "ctx", None):
            self._lib.tsph_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
