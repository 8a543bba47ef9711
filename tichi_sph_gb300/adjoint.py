"""Differentiable rollouts of the DFSPH substep (hand-written adjoint).

The reference has no autodiff.  :class:`DiffRollout` runs ``steps`` substeps of
a scene (each the reference's ``run_step`` substep, ``main.py:347-352``) from
fixed initial positions and a given initial velocity field and viscosity, and
exposes the result -- final positions, velocities and densities -- to
``torch.autograd`` through a custom ``Function`` whose backward calls the CUDA
reverse pass (``tsph_substep_adjoint``, ``tsph_density_adjoint``).

Checkpointing: the forward keeps (positions, velocities) at the start of every
segment of ``checkpoint_every`` substeps and records the last segment on the
tape directly; the backward walks the segments from the end, re-running each
earlier segment from its checkpoint with recording on (one recompute per
substep) and reversing it substep by substep.  Held fixed (not differentiated):
masses, rest densities, the boundary, dt, the solver iteration counts and each
substep's neighbour pairs.
"""
import ctypes as C

import torch

from . import _native
from ._native import check
from .sph import Solver


def _ptr(t, ctype=C.c_float):
    return C.cast(t.data_ptr(), C.POINTER(ctype))


class _Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, v0, mu, sim):
        x, v, rho = sim._forward(v0.detach(), float(mu.detach()))
        ctx.sim = sim
        ctx.v_dtype = v0.dtype
        ctx.mu_dtype = mu.dtype
        return x, v, rho

    @staticmethod
    def backward(ctx, gx, gv, grho):
        gv0, gmu = ctx.sim._backward(gx, gv, grho)
        return gv0.to(ctx.v_dtype), gmu.to(ctx.mu_dtype).reshape(()), None


class DiffRollout:
    """``steps`` substeps of a one-scene DFSPH solver as a differentiable
    function of the initial velocities (``[n, dim]``) and the dynamic viscosity
    (a scalar tensor).  Call it as ``x_T, v_T, rho_T = rollout(v0, mu)``;
    ``rho_T`` is the density at ``x_T`` (the sum ``SPH_prepare_attr``,
    sph.py:50-64, forms)."""

    def __init__(self, config, fluid, bound, steps, checkpoint_every=8, max_iters=8, use_graph=True):
        if steps < 1 or checkpoint_every < 1:
            raise ValueError("steps and checkpoint_every must be positive")
        self.solver = Solver(config, fluid, bound, use_graph=use_graph)
        self.config = config
        self.fluid, self.bound = fluid, bound
        self.device = self.solver.device
        self.steps = int(steps)
        self.K = int(checkpoint_every)
        self.n = int(fluid.part_num[None])
        self.dim = int(config.dim[None])
        self.x0 = fluid.pos[:self.n].detach().clone()
        L = _native.lib()
        self._lib = L
        tape = C.c_void_p()
        with torch.cuda.device(self.device):
            check(L.tsph_tape_create(self.solver.ctx, self.K + 1, int(max_iters), C.byref(tape)), "tsph_tape_create")
        self.tape = tape
        self._density_slot = self.K
        self._ckpt = []
        self._final = None
        # the first divergence-loop test reads the previous solve's compression
        # (main.py:201); it only matters when iter_min is 0
        self._need_compression = int(config.iter_threshold_min[None]) == 0

    # ------------------------------------------------------------------ plumbing
    def _stream(self):
        return C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def _sets(self):
        return C.byref(self.fluid.native_set()), C.byref(self.bound.native_set())

    def _record(self, slot):
        f, b = self._sets()
        check(self._lib.tsph_substep_record(self.solver.ctx, f, b, self.tape, int(slot), self._stream()),
              "tsph_substep_record")

    def _set_start(self, x, v, compression=0.0):
        n = self.n
        self.fluid.pos[:n] = x
        self.fluid.vel[:n] = v
        self.solver.set_state(0.0, 0.0, compression)

    def _compression(self):
        return self.solver.stats()["compression"] if self._need_compression else 0.0

    def segments(self):
        return [(t0, min(t0 + self.K, self.steps)) for t0 in range(0, self.steps, self.K)]

    # ------------------------------------------------------------------ forward / backward
    def _forward(self, v0, mu):
        n = self.n
        with torch.cuda.device(self.device):
            check(self._lib.tsph_set_viscosity(self.solver.ctx, 0, float(mu)), "tsph_set_viscosity")
            self._set_start(self.x0, v0.to(device=self.device, dtype=torch.float32).reshape(n, -1))
            segs = self.segments()
            self._ckpt = []
            for si, (t0, t1) in enumerate(segs):
                last = si == len(segs) - 1
                if not last:
                    self._ckpt.append((self.fluid.pos[:n].clone(), self.fluid.vel[:n].clone(), self._compression()))
                for t in range(t0, t1):
                    if last:
                        self._record(t - t0)
                    else:
                        self.solver.substep()
            rho = torch.empty(n, dtype=torch.float32, device=self.device)
            f, b = self._sets()
            check(self._lib.tsph_density_record(self.solver.ctx, f, b, self.tape, self._density_slot, _ptr(rho),
                                                self._stream()), "tsph_density_record")
            x = self.fluid.pos[:n].clone()
            v = self.fluid.vel[:n].clone()
            self._final = (x.clone(), v.clone())
        return x, v, rho

    def _backward(self, gx, gv, grho):
        n, dev = self.n, self.device
        shape = (n, self.x0.shape[1])
        with torch.cuda.device(dev):
            gx = torch.zeros(shape, dtype=torch.float32, device=dev) if gx is None else \
                gx.to(device=dev, dtype=torch.float32).contiguous().clone()
            gv = torch.zeros(shape, dtype=torch.float32, device=dev) if gv is None else \
                gv.to(device=dev, dtype=torch.float32).contiguous().clone()
            gmu = torch.zeros(1, dtype=torch.float64, device=dev)
            ctx, st = self.solver.ctx, self._stream()
            if grho is not None:
                g = grho.to(device=dev, dtype=torch.float32).contiguous()
                check(self._lib.tsph_density_adjoint(ctx, self.tape, self._density_slot, _ptr(g), _ptr(gx), st),
                      "tsph_density_adjoint")
            segs = self.segments()
            for si in range(len(segs) - 1, -1, -1):
                t0, t1 = segs[si]
                if si != len(segs) - 1:
                    x, v, comp = self._ckpt[si]
                    self._set_start(x, v, comp)
                    for t in range(t0, t1):
                        self._record(t - t0)
                for t in range(t1 - 1, t0 - 1, -1):
                    check(self._lib.tsph_substep_adjoint(ctx, self.tape, t - t0, _ptr(gx), _ptr(gv), _ptr(gx),
                                                         _ptr(gv), _ptr(gmu, C.c_double), st),
                          "tsph_substep_adjoint")
            if self._final is not None:
                self.fluid.pos[:n] = self._final[0]
                self.fluid.vel[:n] = self._final[1]
        return gv, gmu

    def __call__(self, v0, mu):
        if not torch.is_tensor(mu):
            mu = torch.tensor(float(mu), dtype=torch.float64)
        return _Rollout.apply(v0, mu, self)

    def close(self):
        if getattr(self, "tape", None):
            self._lib.tsph_tape_destroy(self.tape)
            self.tape = None
        if getattr(self, "solver", None):
            self.solver.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def com_density_loss(x, rho, mass, rest_density, target, weight=0.1):
    """|centre of mass - target|^2 + weight * mean(((rho - rho0) / rho0)^2)."""
    m = mass.to(x.dtype)
    com = (m[:, None] * x).sum(0) / m.sum()
    e = (rho.to(x.dtype) - rest_density.to(x.dtype)) / rest_density.to(x.dtype)
    return ((com - target.to(x.dtype)) ** 2).sum() + weight * (e * e).mean()
