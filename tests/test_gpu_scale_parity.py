"""One-step parity at the benchmark sizes, from developed flows (needs a GB300).

The golden scenes pin the CUDA path on states of ~100-200 particles a few
substeps after rest.  These tests check the same one-step bar on the benchmark
workloads after the flow has developed (the pressure solves iterate past their
floor where the workload's time step lets them):

1. the CUDA path runs ``develop`` substeps of the workload from rest;
2. its FP32 state (positions, velocities, masses, rest densities / volumes,
   volume fractions) and its carried-over scalars (clock, the compression the
   next divergence test reads) seed the FP64 build of the C restatement of the
   reference (``oracle/sph_port.c`` with REAL=double: every pair term, sum and
   reduction in FP64);
3. both take one substep and are compared.

Tolerances (the one-step bar of the hot-path spec, FP32 against FP64): every
compared field within 1e-5 of its scale max|oracle| (``psi_adv`` is a difference
of the solver's psi, so its scale is psi's: the density for DFSPH, the
compression ratio for VFSPH; with the volume-fraction update ``acce_adv`` is
(v_adv - vel) / dt and is scaled by max|v_adv| / dt); masses and rest densities
2e-6, except with the volume-fraction update, where they are sums of the updated
volume fractions (rho0 = sum_k rho_k vf_k, m = rho0 V) and carry their 1e-5; cell
codes and solver iteration counts exactly equal; dt 1e-6 relative; compression
1e-3 relative; energies 1e-5; the volume-fraction loop's pass count within one
of FP64's and its flags within 1% of the particles of the reference FP32
arithmetic's (a particle whose volume fraction plus its increment lands at ~0
is flagged or not by rounding: in the two-phase state FP64 flags ~0.28M
particles, FP32 ~0.52M, the GPU and the FP32 restatement differing at ~4,400).

One exception, stated with its cause: in the two-phase VFSPH state psi is the
compression ratio (~1) and psi_adv = psi - 1 + ... is ~1e-6 of it, so FP32's
~1e-7 rounding of psi (spline evaluation, reciprocal square root) is a tenth of
psi_adv and of the pressure correction of the velocity.  No FP32 evaluation of
the reference's algorithm meets 1e-5 on velocity there: the FP32 build of the
restatement (the reference's own arithmetic) run from the same state misses it
too, and the test measures that miss.  The velocities (and the velocity
differences built on them, acce_adv and drift_vel) must then be no farther from
the FP64 oracle than 1.5 times the reference arithmetic's own distance (or
within 1e-5); every other field keeps the 1e-5 bar.

Workloads: the 3D dam break of 1,000,000 fluid + 566,742 boundary particles
after 250 substeps, and at five times its time step after 100 substeps (where
the density solve iterates past its floor); the 3D two-phase VFSPH pair of blocks (2,000,000 fluid
particles, surface tension 0.07, volume-fraction update on) after 60 substeps;
the 2D dam break of 5,000 particles after 500 and after 999 substeps (its
stated run is 1,000 substeps).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

STATE = ["pos", "vel", "volume_frac", "rest_volume", "mass", "rest_density"]
FLUID_FIELDS = ["pos", "vel", "vel_adv", "acce_adv", "W", "sph_density", "sph_compression", "psi_adv", "alpha",
                "alpha_1", "alpha_2", "mass", "rest_density"]
BOUND_FIELDS = ["W", "sph_density", "sph_compression", "alpha_2", "alpha"]
TOL = {"mass": 2e-6, "rest_density": 2e-6}


def _need_cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _host(obj, n, keys):
    return {k: getattr(obj, k)[:n].detach().cpu().numpy().copy() for k in keys}


def _err(a, b, scale):
    return float(np.abs(a.astype(np.float64) - b.astype(np.float64)).max(initial=0.0)) / max(scale, 1e-30)


def _one_step_after(cfg_d, scen_d, develop, fbm=False, noise=None, fp32_reference=False):
    """Develops the workload on the GPU, then one substep on the GPU and on the
    FP64 restatement from the same state; returns the worst relative error per
    field and the iteration counts of the compared substep.  With
    ``fp32_reference`` the FP32 build of the restatement also steps from that
    state and its own distance from FP64 is returned as ``info["fp32_ref"]``."""
    from oracle.port import PortSim
    from tichi_sph_gb300 import sph_config
    from tichi_sph_gb300.simulation import Simulation
    cfg = sph_config.Config(cfg_d, scen_d)
    sim = Simulation(cfg, device="cuda", fbm=fbm)
    sim.init_scenario()
    nf, nb = sim.fluid.part_num[None], sim.bound.part_num[None]
    if noise is not None:
        sim.fluid.volume_frac[:nf] = torch.as_tensor(noise(sim.fluid.volume_frac[:nf].cpu().numpy()), device="cuda")
        sim.fluid.update_mass_all()
    solver = sim.solver
    dev_iters = []
    try:
        for _ in range(develop):
            solver.substep()
        st0 = solver.stats()
        dev_iters = (st0["div_iter"], st0["incom_iter"])
        fa, ba = _host(sim.fluid, nf, STATE), _host(sim.bound, nb, STATE)
        port = PortSim(cfg, fa, ba, fbm=fbm, fp64=True)
        try:
            port.set_state(time_count=st0["time_count"], compression=st0["compression"])
            solver.substep()
            gs = solver.stats()
            ps = port.substep()
            P = cfg.phase_num[None]
            fields = list(FLUID_FIELDS) + ["neighb_cell_seq"]
            if float(cfg.surface_tension_gamma[None]) != 0.0:
                fields.append("normal")
            if fbm:
                fields += ["volume_frac", "volume_frac_tmp", "drift_vel", "fbm_zeta"]
            g = _host(sim.fluid, nf, fields)
            gb = _host(sim.bound, nb, BOUND_FIELDS + ["neighb_cell_seq"])
            vfsph = cfg.solver_type == "VFSPH"
            psi = port.fluid.sph_compression if vfsph else port.fluid.sph_density
            psi_scale = float(np.abs(psi).max())
            vmax = float(np.abs(port.fluid.vel_adv).max())
            worst = {}
            for f in fields:
                a, b = g[f], getattr(port.fluid, f).reshape(g[f].shape)
                if f == "neighb_cell_seq":
                    np.testing.assert_array_equal(a, b, err_msg="fluid cell codes")
                    continue
                scale = float(np.abs(b).max(initial=0.0))
                if f == "psi_adv":
                    scale = max(scale, psi_scale)
                if fbm and f == "acce_adv":
                    scale = max(scale, vmax / ps["dt"])
                if fbm and f == "drift_vel":
                    scale = max(scale, vmax)
                if f == "volume_frac_tmp":
                    scale = max(scale, float(np.abs(port.fluid.volume_frac).max()))
                worst["fluid " + f] = _err(a, b, scale)
            for f in BOUND_FIELDS:
                b = getattr(port.bound, f).reshape(gb[f].shape)
                worst["bound " + f] = _err(gb[f], b, float(np.abs(b).max(initial=0.0)))
            np.testing.assert_array_equal(gb["neighb_cell_seq"], port.bound.neighb_cell_seq, err_msg="bound cells")
            assert P >= 1
            info = {"develop_iters": dev_iters, "iters": (gs["div_iter"], gs["incom_iter"]),
                    "port_iters": (ps["div_iter"], ps["incom_iter"]), "fbm": (gs["fbm_passes"], ps["fbm_passes"]),
                    "dt": (gs["dt"], ps["dt"]), "compression": (gs["compression"], ps["compression"]),
                    "ke": (gs["kinetic_energy"], ps["kinetic_energy"]),
                    "pe": (gs["potential_energy"], ps["potential_energy"]), "n": (nf, nb)}
            if fp32_reference:
                p32 = PortSim(cfg, fa, ba, fbm=fbm, fp64=False)
                try:
                    p32.set_state(time_count=st0["time_count"], compression=st0["compression"])
                    info["fp32_ref_fbm"] = p32.substep()["fbm_passes"]
                    if fbm:
                        gflag = sim.fluid.flag[:nf].cpu().numpy() != 0
                        info["flag_diff_fp32"] = float(np.mean(gflag != (p32.fluid.flag != 0)))
                        info["flag_diff_fp64"] = float(np.mean(gflag != (port.fluid.flag != 0)))
                    ref = {}
                    for f in ("vel", "acce_adv", "drift_vel"):
                        if f == "drift_vel" and not fbm:
                            continue
                        b = getattr(port.fluid, f)
                        scale = float(np.abs(b).max())
                        if fbm and f == "acce_adv":
                            scale = max(scale, vmax / ps["dt"])
                        if f == "drift_vel":
                            scale = max(scale, vmax)
                        ref[f] = _err(getattr(p32.fluid, f), b, scale)
                    info["fp32_ref"] = ref
                finally:
                    p32.close()
            print("one step after %d substeps (%d fluid, %d boundary): %s" % (develop, nf, nb, info))
            print("worst relative errors: %s" % {k: "%.2e" % v for k, v in sorted(worst.items())})
            return worst, info
        finally:
            port.close()
    finally:
        solver.close()


def _check(worst, info, fbm=False):
    assert info["iters"] == info["port_iters"], info
    if fbm:
        # a particle whose volume fraction plus its increment sits at ~0 is
        # flagged or not by rounding (in the two-phase state a quarter of the
        # particles do: FP64 flags ~0.28M where FP32 flags ~0.52M), which may add
        # or save a pass: the count within one of FP64's, and the flags within
        # 1% of the particles of the reference FP32 arithmetic's
        assert abs(info["fbm"][0] - info["fbm"][1]) <= 1, info
        if "flag_diff_fp32" in info:
            assert info["flag_diff_fp32"] <= 0.01, info
    assert info["dt"][0] == pytest.approx(info["dt"][1], rel=1e-6)
    assert info["compression"][0] == pytest.approx(info["compression"][1], rel=1e-3, abs=1e-7)
    assert info["ke"][0] == pytest.approx(info["ke"][1], rel=1e-5)
    assert info["pe"][0] == pytest.approx(info["pe"][1], rel=1e-5)
    ref = info.get("fp32_ref", {})
    for k, v in worst.items():
        f = k.split(" ", 1)[1]
        tol = 1e-5 if fbm else TOL.get(f, 1e-5)
        if k.startswith("fluid ") and f in ("vel", "vel_adv", "acce_adv", "drift_vel") and ref:
            tol = max(tol, 1.5 * ref["vel" if f == "vel_adv" else f])
        assert v <= tol, "%s rel err %.3g > %.3g (%s)" % (k, v, tol, info)


def test_dambreak_3d_1m_developed_one_step():
    """3D DFSPH dam break, 1,000,000 fluid + 566,742 boundary particles (the
    headline workload) after 250 substeps, the column compressed under its
    weight.  At this workload's time step (2e-4 s) both solves stay at their
    floor of two iterations (measured over 1,500 substeps from rest: the
    compression after the density solve stays below 2e-4, under its 1e-3
    tolerance)."""
    _need_cuda()
    from tichi_sph_gb300 import workloads
    cfg_d, scen_d = workloads.dambreak_3d(100)
    worst, info = _one_step_after(cfg_d, scen_d, 250)
    _check(worst, info)
    assert info["compression"][1] > 0.0, info


def test_dambreak_3d_1m_iterating_one_step():
    """The same 1M dam break at a five times larger time step (solver_cs 10:
    dt 1e-3), after 100 substeps: the density solve iterates past its floor, so
    the compared substep runs the Jacobi iterations the benchmark's own time
    step does not reach."""
    _need_cuda()
    from tichi_sph_gb300 import workloads
    cfg_d, scen_d = workloads.dambreak_3d(100)
    cfg_d["solver_cs"] = 10
    worst, info = _one_step_after(cfg_d, scen_d, 100)
    _check(worst, info)
    assert info["iters"][1] > int(cfg_d["solver_iter_threshold_min"]), info


def test_twophase_3d_2m_developed_one_step():
    """3D two-phase VFSPH, two 1 m blocks of 1,000,000 particles each (rest
    densities 1000 / 500, seeded volume-fraction noise), surface tension 0.07
    and the volume-fraction update on, after 60 substeps."""
    _need_cuda()
    from tichi_sph_gb300 import workloads
    cfg_d, scen_d, noise = workloads.twophase_3d()
    worst, info = _one_step_after(cfg_d, scen_d, 60, fbm=True, noise=noise, fp32_reference=True)
    _check(worst, info, fbm=True)


@pytest.mark.parametrize("develop", [500, 999])
def test_dambreak_2d_developed_one_step(develop):
    """2D DFSPH dam break, 5,000 fluid particles, after 500 and after 999
    substeps: the compared substep is the 501st / the 1,000th."""
    _need_cuda()
    from tichi_sph_gb300 import workloads
    cfg_d, scen_d = workloads.dambreak_2d()
    worst, info = _one_step_after(cfg_d, scen_d, develop)
    _check(worst, info)
