"""The density sweep that allocates nothing, against the solver step (needs a GPU).

``tsph_fluid_density_noalloc`` serves callers that cannot allocate device memory
where they call in (a host that pre-plans all device memory, or an allocator
that owns the device) and therefore cannot create a solver context.  Its W /
sph_density / sph_compression must equal those the regular step
(``tsph_substep``) computes from the same positions, within the one-step
tolerance of the parity tests (1e-5 of each field's scale) -- on two calls in a
row, so a call that leaves stale data in the shared scratch array would show.
Kept in a file collected last (name starts with test_zz_).
"""
import ctypes

import numpy as np
import pytest
import torch

from tests import golden_io as G
from tichi_sph_gb300 import Fluid, Solver, _native, sph_config

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _fp(t):
    return ctypes.cast(t.data_ptr(), _native._fp)


def _setup(scene):
    cfg = sph_config.load(*G.paths(scene))
    init, _ = G.load(scene)
    sets = []
    for uid, name in enumerate(("fluid", "bound")):
        cap = cfg.fluid_max_part_num[None] if uid == 0 else cfg.bound_max_part_num[None]
        o = Fluid(cap, cfg, uid, device="cuda")
        n = int(init[name + "_n"])
        o.part_num[None] = n
        for k in G.STATE_IN:
            getattr(o, k)[:n] = torch.as_tensor(init[name + "_" + k], device="cuda").reshape(getattr(o, k)[:n].shape)
        sets.append(o)
    return cfg, sets[0], sets[1]


def _noalloc(cfg, fl, bd, pos, mass, rv):
    L = _native.lib()
    nf, nb = fl.part_num[None], bd.part_num[None]
    W = torch.full((nf,), -1.0, device="cuda")
    rho = torch.full((nf,), -1.0, device="cuda")
    comp = torch.full((nf,), -1.0, device="cuda")
    params = cfg.to_params()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = L.tsph_fluid_density_noalloc(ctypes.byref(params), _fp(pos), _fp(mass), _fp(rv), nf,
                                      _fp(bd.pos), _fp(bd.mass), _fp(bd.rest_volume), nb,
                                      _fp(W), _fp(rho), _fp(comp), stream)
    _native.check(rc, "tsph_fluid_density_noalloc")
    torch.cuda.synchronize()
    return W, rho, comp


def _close(a, b, name):
    a = a.cpu().numpy().astype(np.float64)
    b = b.cpu().numpy().astype(np.float64)
    scale = max(float(np.abs(b).max()), 1e-30)
    err = float(np.abs(a - b).max()) / scale
    assert err <= TOL, "%s: rel err %.3g" % (name, err)


@pytest.mark.parametrize("scene", ["dfsph3d", "vfsph2d", "edge2d"])
def test_noalloc_density_matches_step_two_calls(scene):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    cfg, fl, bd = _setup(scene)
    solver = Solver(cfg, fl, bd, fbm=scene in G.FBM_SCENES)
    nf = fl.part_num[None]
    for call in range(2):
        # inputs of the step's density sweep: positions and masses before the step
        pos = fl.pos[:nf].clone()
        mass = fl.mass[:nf].clone()
        rv = fl.rest_volume[:nf].clone()
        solver.substep()
        solver.stats()
        W, rho, comp = _noalloc(cfg, fl, bd, pos, mass, rv)
        _close(W, fl.W[:nf], "W call %d" % call)
        _close(rho, fl.sph_density[:nf], "sph_density call %d" % call)
        _close(comp, fl.sph_compression[:nf], "sph_compression call %d" % call)
    solver.close()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    cfg, fl, bd = _setup("dfsph2d")
    params = cfg.to_params()
    params.node_num = 131072 + 1
    L = _native.lib()
    z = _fp(fl.pos)
    rc = L.tsph_fluid_density_noalloc(ctypes.byref(params), z, z, z, 10, z, z, z, 10, z, z, z, None)
    assert rc == _native.ERR_CAPACITY
    assert b"TSPH_NOALLOC_MAX_CELLS" in L.tsph_last_error()
    params = cfg.to_params()
    rc = L.tsph_fluid_density_noalloc(ctypes.byref(params), z, z, z, 65536 + 1, z, z, z, 10, z, z, z, None)
    assert rc == _native.ERR_CAPACITY
    assert b"TSPH_NOALLOC_MAX_PARTICLES" in L.tsph_last_error()
