"""The step's status path under host-injected faults (needs a GPU; no GPU fault
is provoked: the faults are configurations and inputs set from the host).

* Iteration caps (main.py:212-213, 233-234): solver_iter_threshold_max 0 and 1
  with tolerances no solve can reach.  Each solve stops after iter_max + 1
  iterations (at least one: the floor of two is cut by the cap), the step sets
  TSPH_ST_DIV_ITER_CAP and TSPH_ST_DENS_ITER_CAP and reports them once as
  RuntimeWarnings, and iteration counts and fields equal the FP64 oracle's.
* A non-finite position (one fluid particle's x set to NaN from the host): the
  step completes and sets TSPH_ST_NONFINITE_POS; the particle has no cell, so it
  is nobody's neighbour, and every other particle equals the oracle run without
  it.  Both solves run a fixed two iterations here (unreachable tolerances,
  iter_max 1), so the loop decisions do not depend on the mean compression,
  which the extra particle would change.
"""
import json

import numpy as np
import pytest
import torch

from oracle import sph_oracle as O
from tests import golden_io as G
from tichi_sph_gb300 import _native

pytestmark = pytest.mark.gpu

SCENE = "dfsph3d"
FIELDS = ("pos", "vel", "vel_adv", "sph_density", "psi_adv", "alpha", "W")


def _need_cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _config(iter_max, unreachable=True):
    cpath, spath = G.paths(SCENE)
    cfg_d, scen_d = json.load(open(cpath)), json.load(open(spath))
    cfg_d["solver_iter_threshold_max"] = iter_max
    if unreachable:
        cfg_d["solver_divergence_threshold"] = 1e-12
        cfg_d["solver_compression_threshold"] = 1e-12
    return cfg_d, scen_d


def _gpu(cfg_d, scen_d, fa, ba, use_graph=True):
    from tichi_sph_gb300 import Fluid, Solver, sph_config
    cfg = sph_config.Config(cfg_d, scen_d)
    objs = []
    for uid, (cap, arrs) in enumerate(((cfg.fluid_max_part_num[None], fa), (cfg.bound_max_part_num[None], ba))):
        o = Fluid(cap, cfg, uid, device="cuda")
        n = len(arrs["pos"])
        o.part_num[None] = n
        for k, v in arrs.items():
            getattr(o, k)[:n] = torch.as_tensor(np.asarray(v, np.float32), device="cuda").reshape(getattr(o, k)[:n].shape)
        objs.append(o)
    return objs[0], objs[1], Solver(cfg, objs[0], objs[1], use_graph=use_graph)


def _oracle(cfg_d, scen_d, fa, ba):
    p = O.Params.from_config(cfg_d, scen_d, taichi_f32=True)
    f64 = lambda d: {k: np.asarray(v, np.float32).astype(np.float64) for k, v in d.items()}
    fl, bd = O.sets_from_arrays(p, f64(fa), f64(ba))
    st = O.run_substep(fl, bd, p, O.Stats())
    return fl, st


def _compare(gfl, ofl, keep=None, tol=1e-5):
    dens = float(np.abs(ofl.sph_density).max())
    for f in FIELDS:
        a = getattr(gfl, f)[:gfl.part_num[None]].cpu().numpy().astype(np.float64)
        if keep is not None:
            a = a[keep]
        b = np.asarray(getattr(ofl, f), np.float64).reshape(a.shape)
        scale = max(float(np.abs(b).max()), dens if f == "psi_adv" else 0.0)
        err = float(np.abs(a - b).max()) / scale
        assert err <= tol, (f, err)


@pytest.mark.parametrize("use_graph", [True, False], ids=["graph", "hostloop"])
@pytest.mark.parametrize("iter_max", [0, 1])
def test_iteration_cap_sets_status_and_matches_oracle(iter_max, use_graph):
    _need_cuda()
    init, _ = G.load(SCENE)
    fa, ba = G.init_arrays(init, "fluid"), G.init_arrays(init, "bound")
    cfg_d, scen_d = _config(iter_max)
    gfl, gbd, solver = _gpu(cfg_d, scen_d, fa, ba, use_graph)
    try:
        solver.substep()
        with pytest.warns(RuntimeWarning) as rec:
            st = solver.stats()
        msgs = " ".join(str(w.message) for w in rec)
        assert "divergence-free solve stopped" in msgs and "constant-density solve stopped" in msgs
        bits = _native.ST_DIV_ITER_CAP | _native.ST_DENS_ITER_CAP
        assert st["status"] & bits == bits
        ofl, ost = _oracle(cfg_d, scen_d, fa, ba)
        assert (st["div_iter"], st["incom_iter"]) == (ost.div_iter, ost.incom_iter) == (iter_max + 1, iter_max + 1)
        _compare(gfl, ofl)
        solver.substep()
        st2 = solver.stats()   # reported once per condition: no second warning
        assert st2["status"] & bits == bits
    finally:
        solver.close()


def test_nonfinite_position_sets_status_and_leaves_the_rest_exact():
    _need_cuda()
    init, _ = G.load(SCENE)
    fa, ba = G.init_arrays(init, "fluid"), G.init_arrays(init, "bound")
    cfg_d, scen_d = _config(1)
    k = len(fa["pos"]) // 2
    bad = {key: np.array(v, copy=True) for key, v in fa.items()}
    bad["pos"] = bad["pos"].astype(np.float32)
    bad["pos"][k, 0] = np.nan
    gfl, gbd, solver = _gpu(cfg_d, scen_d, bad, ba)
    try:
        solver.substep()
        with pytest.warns(RuntimeWarning, match="not finite"):
            st = solver.stats()
        assert st["status"] & _native.ST_NONFINITE_POS
        assert st["fluid_in_grid"] == len(fa["pos"]) - 1
        keep = np.arange(len(fa["pos"])) != k
        ofl, ost = _oracle(cfg_d, scen_d, {key: v[keep] for key, v in fa.items()}, ba)
        assert (st["div_iter"], st["incom_iter"]) == (ost.div_iter, ost.incom_iter) == (2, 2)
        _compare(gfl, ofl, keep=keep)
        assert np.isnan(gfl.pos[k, 0].item())
    finally:
        solver.close()
