"""Run-time emission on the GPU against the reference's own run (needs a GPU).

The golden scene ``inlet3d`` (``tests/golden/make_golden.py``) was run through
the reference's emitters and its scenario schedule (main.py:26-112: an inlet
pushing 3 x 3 particles at 7 m/s every ~2.85 ms until 6.5 ms, a boundary cube
appearing at 1.5 ms and a fluid cube at 4.5 ms, each substep starting with
refresh_scenario, main.py:346).  ``Simulation.substep`` replays the same
schedule and steps the CUDA path across every emission: the particle counts
change between substeps, so each emission rebuilds the native set views,
re-captures the substep's CUDA graph (graph mode) and, for the boundary cube,
drops the kept boundary-boundary sums.  After every substep the particle counts
equal the reference's and the fields agree with the reference's FP64 run within
10x the one-step tolerance (the chained-trajectory bar of the parity tests).
A capacity too small for an emission is reported as the reference reports a
failed emission (a warning, and the object or inlet is dropped); a set larger
than the context's capacity is refused before any launch.
"""
import numpy as np
import pytest
import torch

from tests import golden_io as G

pytestmark = pytest.mark.gpu

TOL = 1e-4   # 10 x the one-step tolerance, as for chained trajectories
FLUID = ("pos", "vel", "sph_density", "psi_adv", "alpha", "W")
BOUND = ("W", "sph_density", "alpha")


def _need_cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _sim(use_graph=True, fluid_cap=None):
    import json
    from tichi_sph_gb300 import sph_config
    from tichi_sph_gb300.simulation import Simulation
    cpath, spath = G.paths("inlet3d")
    cfg_d, scen_d = json.load(open(cpath)), json.load(open(spath))
    if fluid_cap is not None:
        scen_d["fluid"]["max_part_num"] = fluid_cap
    sim = Simulation(sph_config.Config(cfg_d, scen_d), device="cuda", use_graph=use_graph)
    sim.init_scenario()
    return sim


@pytest.mark.parametrize("use_graph", [True, False], ids=["graph", "hostloop"])
def test_emission_across_substeps_matches_reference(use_graph):
    _need_cuda()
    init, gold = G.load("inlet3d")
    sim = _sim(use_graph)
    try:
        for name, obj in (("fluid", sim.fluid), ("bound", sim.bound)):
            n = int(init[name + "_n"])
            assert obj.part_num[None] == n
            for k in G.STATE_IN:
                a = getattr(obj, k)[:n].cpu().numpy()
                np.testing.assert_array_equal(a, init[name + "_" + k].reshape(a.shape), err_msg=name + " " + k)
        counts = []
        for step in range(G.n_steps(gold)):
            st = sim.substep()
            p = "s%d_" % step
            nf, nb = sim.fluid.part_num[None], sim.bound.part_num[None]
            counts.append((nf, nb))
            assert (nf, nb) == (len(gold[p + "fluid_pos"]), len(gold[p + "bound_pos"])), step
            assert (st["div_iter"], st["incom_iter"]) == (int(gold[p + "div_iter"]), int(gold[p + "incom_iter"]))
            assert st["time_count"] == pytest.approx(float(gold[p + "time_count"]), rel=1e-6)
            dens = float(np.abs(gold[p + "fluid_sph_density"]).max())
            for name, obj, fields, n in (("fluid", sim.fluid, FLUID, nf), ("bound", sim.bound, BOUND, nb)):
                for f in fields:
                    a = getattr(obj, f)[:n].cpu().numpy().astype(np.float64)
                    b = np.asarray(gold[p + name + "_" + f], dtype=np.float64).reshape(a.shape)
                    scale = max(float(np.abs(b).max()), dens if f == "psi_adv" else 0.0)
                    err = float(np.abs(a - b).max()) / scale
                    assert err <= TOL, "step %d %s %s rel err %.3g" % (step, name, f, err)
        # the schedule really emitted: inlet pushes at steps 0, 3, 6, the boundary cube at 2, the fluid cube at 5
        assert counts[0][0] == 134 and counts[2][1] > counts[1][1] and counts[5][0] == counts[4][0] + 27
        assert counts[-1][0] == 179
    finally:
        sim.solver.close()


def test_emission_beyond_capacity_warns_and_drops_the_object():
    """With room for one inlet push only, the later pushes and the delayed fluid
    cube fail as the reference's refresh_scenario reports a failed emission
    (main.py:97-99, 108-110): a warning, the inlet or object dropped, the run
    going on with the particles it has."""
    _need_cuda()
    sim = _sim(fluid_cap=140)
    try:
        with pytest.warns(RuntimeWarning) as rec:
            for _ in range(8):
                sim.substep()
        msgs = " ".join(str(w.message) for w in rec)
        assert "refresh_inlets failed" in msgs and "invalid scenario object" in msgs
        assert sim.fluid.part_num[None] == 134 and not sim.inlets and not sim.scenario_wait_buffer
        assert np.isfinite(sim.fluid.pos[:134].cpu().numpy()).all()
    finally:
        sim.solver.close()


def test_set_beyond_context_capacity_is_refused():
    """A particle count above the capacity the context was created with is
    refused with TSPH_ERR_CAPACITY before any kernel runs."""
    _need_cuda()
    from tichi_sph_gb300._native import TsphError
    sim = _sim()
    try:
        sim.substep()
        cap = sim.fluid.max_part_num
        sim.fluid.part_num[None] = cap + 1
        with pytest.raises(TsphError, match="code 2"):
            sim.solver.substep()
        sim.fluid.part_num[None] = 134
        sim.solver.substep()   # the context is still usable
        assert np.isfinite(sim.fluid.pos[:134].cpu().numpy()).all()
    finally:
        sim.solver.close()
