"""Long run of the 2D dam break (5,000 fluid particles at 0.02 m, dt 1e-3,
density tolerance 0.1%): the CUDA path against the C restatement of the
reference (FP32, the reference's kernel order; oracle/sph_port.c) over 600
substeps (0.6 s, the front crossing most of the tank).  Checked every 25
substeps (needs a GPU):

* mass conservation: the fluid's total mass is exactly that of the initial
  state, in both runs;
* mean density error: the compression after each density solve stays within
  the solver's tolerance (or the solve hit its iteration cap), and the run's
  mean compression agrees with the restatement's within 5%;
* dam-break front (largest x of the fluid): within 0.01 m (half a particle
  spacing) for the first 300 substeps and within 0.04 m (two spacings) after,
  where the two FP32 runs' different summation orders have grown into
  particle-scale differences at the front; the fluid's mean height within
  1e-3 m throughout.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _need_cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def test_dambreak_2d_long_run_against_the_restatement():
    _need_cuda()
    from oracle.port import PortSim
    from tichi_sph_gb300 import Solver, sph_config, workloads
    from tichi_sph_gb300.simulation import Simulation
    cfg_d, scen_d = workloads.dambreak_2d()
    cfg = sph_config.Config(cfg_d, scen_d)
    sim = Simulation(cfg, device="cuda")
    sim.init_scenario()
    nf, nb = sim.fluid.part_num[None], sim.bound.part_num[None]
    keys = ["pos", "vel", "volume_frac", "rest_volume", "mass", "rest_density"]
    fa = {k: getattr(sim.fluid, k)[:nf].cpu().numpy() for k in keys}
    ba = {k: getattr(sim.bound, k)[:nb].cpu().numpy() for k in keys}
    solver = Solver(cfg, sim.fluid, sim.bound)
    port = PortSim(cfg, fa, ba)
    tol = float(cfg_d["solver_compression_threshold"])
    iter_max = int(cfg_d["solver_iter_threshold_max"])
    m0 = float(np.asarray(fa["mass"], dtype=np.float64).sum())
    comp_g, comp_p = [], []
    try:
        for step in range(1, 601):
            solver.substep()
            gs = solver.stats()
            ps = port.substep()
            assert gs["time_count"] == pytest.approx(ps["time_count"], rel=1e-6)
            for st in (gs, ps):
                assert st["compression"] <= tol or st["incom_iter"] > iter_max, (step, st)
            comp_g.append(gs["compression"])
            comp_p.append(ps["compression"])
            if step % 25:
                continue
            gp = sim.fluid.pos[:nf].cpu().numpy().astype(np.float64)
            pp = port.fluid.pos.astype(np.float64)
            front_tol = 0.01 if step <= 300 else 0.04
            assert abs(gp[:, 0].max() - pp[:, 0].max()) <= front_tol, (step, gp[:, 0].max(), pp[:, 0].max())
            assert abs(gp[:, 1].mean() - pp[:, 1].mean()) <= 1e-3, step
        assert float(sim.fluid.mass[:nf].double().sum()) == m0
        assert float(port.fluid.mass.astype(np.float64).sum()) == m0
        assert np.mean(comp_g) == pytest.approx(np.mean(comp_p), rel=0.05)
    finally:
        solver.close()
        port.close()
