"""Kernel-level composition of the step against the fused step (needs a GPU).

A caller can write ``sph_step`` as the reference's ``main.py:175-256`` does, from
the reference-named kernels of ``tichi_sph_gb300.sph`` with Python solver loops
that read ``fluid.compression[None]``, or with the phase entries of the C ABI
(``tsph_grid_build`` ... ``tsph_update``, whole loops by ``tsph_solve``).  The
same kernels then run in the same order as in the fused ``tsph_substep``, so
every particle field and every step scalar must be bitwise equal to the fused
step's, substep after substep (golden scenes: DFSPH 3D, VFSPH 2D with surface
tension and the volume-fraction update, and the weakly compressible block).
Leaving a force out of the composed step equals the fused step with that
force's coefficient zero, bit for bit; calls out of order are errors.
"""
import json

import numpy as np
import pytest
import torch

from tests import golden_io as G
from tichi_sph_gb300 import sph as S
from tichi_sph_gb300._native import TsphError

pytestmark = pytest.mark.gpu

FIELDS = ["pos", "vel", "vel_adv", "acce_adv", "mass", "rest_density", "volume_frac", "W", "sph_density",
          "sph_compression", "psi_adv", "alpha", "alpha_1", "alpha_2", "normal", "flag", "neighb_cell_seq",
          "neighb_in_cell_seq", "pressure", "volume_frac_tmp", "drift_vel", "fbm_zeta"]
SCALARS = ["dt", "time_count", "compression", "kinetic_energy", "potential_energy", "div_iter", "incom_iter",
           "fbm_passes", "status"]


def _need_cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _make(scene, cfg_d=None, scen_d=None):
    from tichi_sph_gb300 import Fluid, Ngrid, Solver, sph_config
    if cfg_d is None:
        cfg = sph_config.load(*G.paths(scene))
    else:
        cfg = sph_config.Config(cfg_d, scen_d)
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
    ngrid = Ngrid(cfg)
    solver = Solver(cfg, sets[0], sets[1], fbm=scene in G.FBM_SCENES, wcsph=scene in G.WC_SCENES, ngrid=ngrid)
    return cfg, ngrid, sets[0], sets[1], solver


def reference_shaped_sph_step(config, ngrid, fluid, bound, fbm=False, wc=False, viscosity=True):
    """main.py:175-256, call for call (its commented-out blocks switched by fbm / wc)."""
    ngrid.clear_node()
    ngrid.encode(fluid)
    ngrid.encode(bound)
    ngrid.mem_shift()
    ngrid.fill_node(fluid)
    ngrid.fill_node(bound)
    S.SPH_clean_value(fluid)
    S.SPH_clean_value(bound)
    S.SPH_prepare_attr(ngrid, fluid, fluid)
    S.SPH_prepare_attr(ngrid, fluid, bound)
    S.SPH_prepare_attr(ngrid, bound, bound)
    S.SPH_prepare_attr(ngrid, bound, fluid)
    S.SPH_prepare_alpha_1(ngrid, fluid, fluid)
    S.SPH_prepare_alpha_1(ngrid, fluid, bound)
    S.SPH_prepare_alpha_2(ngrid, fluid, fluid)
    S.SPH_prepare_alpha_2(ngrid, bound, fluid)
    S.SPH_prepare_alpha(fluid)
    S.SPH_prepare_alpha(bound)
    div_iter = 0
    S.SPH_vel_2_vel_adv(fluid)
    while div_iter < config.iter_threshold_min[None] or fluid.compression[None] > config.divergence_threshold[None]:
        S.IPPE_adv_psi_init(fluid)
        S.IPPE_adv_psi(ngrid, fluid, fluid)
        S.IPPE_adv_psi(ngrid, fluid, bound)
        S.IPPE_psi_adv_non_negative(fluid)
        S.IPPE_update_vel_adv(ngrid, fluid, fluid)
        S.IPPE_update_vel_adv(ngrid, fluid, bound)
        div_iter += 1
        if div_iter > config.iter_threshold_max[None]:
            break
    S.SPH_vel_adv_2_vel(fluid)
    S.SPH_advection_gravity_acc(fluid)
    if viscosity:
        S.SPH_advection_viscosity_acc(ngrid, fluid, fluid)
    S.SPH_advection_surface_tension_acc(ngrid, fluid, fluid)
    S.SPH_advection_update_vel_adv(fluid)
    incom_iter = 0
    while incom_iter < config.iter_threshold_min[None] or fluid.compression[None] > config.compression_threshold[None]:
        S.IPPE_adv_psi_init(fluid)
        S.IPPE_adv_psi(ngrid, fluid, fluid)
        S.IPPE_adv_psi(ngrid, fluid, bound)
        S.IPPE_psi_adv_non_negative(fluid)
        S.IPPE_update_vel_adv(ngrid, fluid, fluid)
        S.IPPE_update_vel_adv(ngrid, fluid, bound)
        incom_iter += 1
        if incom_iter > config.iter_threshold_max[None]:
            break
    if wc:
        S.WC_pressure_val(fluid)
        S.WC_pressure_acce(ngrid, fluid, fluid)
        S.WC_pressure_acce(ngrid, fluid, bound)
        S.SPH_advection_update_vel_adv(fluid)
    if fbm:
        while fluid.general_flag[None] > 0:
            S.SPH_FBM_clean_tmp(fluid)
            S.SPH_FBM_convect(ngrid, fluid, fluid)
            S.SPH_FBM_diffuse(ngrid, fluid, fluid)
            S.SPH_FBM_check_tmp(fluid)
        S.SPH_update_volume_frac(fluid)
    S.SPH_update_mass(fluid)
    S.SPH_update_pos(fluid)
    S.SPH_update_energy(fluid)
    return div_iter, incom_iter


def phase_entry_sph_step(solver, fbm=False, wc=False):
    """The same step through the phase entries, whole loops by tsph_solve."""
    from tichi_sph_gb300 import _native
    solver.grid_build()
    solver.density_alpha()
    kd, _ = solver.solve(_native.SOLVE_DIV)
    solver.nonpressure()
    kp, _ = solver.solve(_native.SOLVE_DENS)
    if wc:
        solver.wc_pressure()
    if fbm:
        while solver.fbm_pass():
            pass
    solver.update()
    return kd, kp


def _state(fl, bd, solver):
    nf, nb = fl.part_num[None], bd.part_num[None]
    out = {"fluid " + k: getattr(fl, k)[:nf].cpu().numpy().copy() for k in FIELDS}
    out.update({"bound " + k: getattr(bd, k)[:nb].cpu().numpy().copy()
                for k in ("W", "sph_density", "sph_compression", "alpha", "alpha_2", "neighb_cell_seq")})
    st = solver.stats()
    out.update({"stat " + k: st[k] for k in SCALARS})
    return out


def _assert_same(a, b, what):
    assert a.keys() == b.keys()
    for k in a:
        np.testing.assert_array_equal(np.asarray(a[k]), np.asarray(b[k]), err_msg="%s: %s" % (what, k))


@pytest.mark.parametrize("how", ["reference_kernels", "phase_entries"])
@pytest.mark.parametrize("scene", ["dfsph3d", "vfsph2d", "wcsph2d"])
def test_composed_step_equals_fused_step(scene, how):
    _need_cuda()
    fbm, wc = scene in G.FBM_SCENES, scene in G.WC_SCENES
    cfg, ngrid, fl, bd, composed = _make(scene)
    _, _, fl2, bd2, fused = _make(scene)
    try:
        for step in range(3):
            S.cfl_condition(fl)   # run_step's substep: cfl_condition, then sph_step (main.py:347-350)
            if how == "reference_kernels":
                iters = reference_shaped_sph_step(cfg, ngrid, fl, bd, fbm=fbm, wc=wc)
            else:
                iters = phase_entry_sph_step(composed, fbm=fbm, wc=wc)
            fused.substep()
            a, b = _state(fl, bd, composed), _state(fl2, bd2, fused)
            assert iters == (b["stat div_iter"], b["stat incom_iter"]), (step, iters)
            _assert_same(a, b, "%s %s step %d" % (scene, how, step))
    finally:
        composed.close()
        fused.close()


def test_force_left_out_equals_zero_coefficient():
    """A composed step without SPH_advection_viscosity_acc equals the fused step
    of the same scene with global_dynamic_viscosity 0, bit for bit."""
    _need_cuda()
    scene = "dfsph3d"
    cpath, spath = G.paths(scene)
    cfg_d, scen_d = json.load(open(cpath)), json.load(open(spath))
    cfg, ngrid, fl, bd, composed = _make(scene)
    scen0 = json.loads(json.dumps(scen_d))
    scen0["sim_env"]["global_dynamic_viscosity"] = 0.0
    _, _, fl2, bd2, fused = _make(scene, cfg_d, scen0)
    try:
        for step in range(2):
            S.cfl_condition(fl)
            reference_shaped_sph_step(cfg, ngrid, fl, bd, viscosity=False)
            fused.substep()
            _assert_same(_state(fl, bd, composed), _state(fl2, bd2, fused), "no viscosity, step %d" % step)
    finally:
        composed.close()
        fused.close()


def test_out_of_order_calls_raise():
    _need_cuda()
    from tichi_sph_gb300 import _native
    cfg, ngrid, fl, bd, solver = _make("dfsph3d")
    try:
        # a group left incomplete: the fused density sweep has the fluid-boundary pairs
        ngrid.clear_node()
        ngrid.encode(fl)
        ngrid.encode(bd)
        ngrid.mem_shift()
        ngrid.fill_node(fl)
        ngrid.fill_node(bd)
        S.SPH_clean_value(fl)
        S.SPH_clean_value(bd)
        S.SPH_prepare_attr(ngrid, fl, fl)
        with pytest.raises(TsphError, match="SPH_prepare_attr\\(fb\\)"):
            S.IPPE_adv_psi_init(fl)
        # the C entries refuse a phase out of order (the grid was built, density not run)
        with pytest.raises(TsphError, match="code 4"):
            solver.nonpressure()
        with pytest.raises(TsphError, match="code 4"):
            solver.update_vel_adv(_native.SOLVE_DIV)
        solver.density_alpha()
        with pytest.raises(TsphError, match="code 4"):
            solver.update_vel_adv(_native.SOLVE_DIV)   # a sweep B before its sweep A
        with pytest.raises(TsphError, match="code 4"):
            solver.adv_psi(_native.SOLVE_DENS)          # the density solve before the non-pressure forces
        with pytest.raises(TsphError, match="code 1"):
            solver.fbm_pass()                           # the context has no volume-fraction update
    finally:
        solver.close()
