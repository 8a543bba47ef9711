#!/usr/bin/env python
"""Throughput of the SPH substep (particle-steps/s) on the GPU, and the reference arm.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload: the 3D single-phase DFSPH dam break (``workloads.dambreak_3d``): a
1 m cube of 1,000,000 fluid particles at 0.01 m in a 3 x 1.5 x 1 m tank of
566,742 boundary particles, h = 0.02, dt <= 2e-4 (CFL), density tolerance 0.1%,
divergence tolerance 1%, 500 substeps from rest.  A step is one substep of the
reference's ``run_step`` (``cfl_condition`` + ``sph_step``, main.py:347-352) over
the whole scene; the metric counts fluid particles only (particle-steps/s =
fluid particles x substeps / time; boundary particles are not counted).  The
timed window is the end of the 500-substep run: the flow first develops for
500 - W - K untimed substeps (``--develop``), then W warm-up and K timed
substeps follow: the developed flow (the column collapsed and running along
the floor), not the lattice right after rest.  At this time step the pressure
solves still converge at their floor of two iterations each; the extra entry
``dambreak3d_cs10`` times the same scene at a five times larger step, where
they iterate.

The same line carries the other workloads of the hot path, each timed with CUDA
events at N = 1: ``batched`` (256 dam breaks of uneven size in one launch
against the same scenes stepped one at a time), ``twophase3d`` (2M-particle
two-phase VFSPH with surface tension and the volume-fraction update, the end of
its 300-substep run), ``dambreak2d`` (5,000-particle 2D dam break, substeps 4 to
1,000 of its run), ``dambreak3d_cs10`` (the headline scene at solver_cs 10, the
last 20 of 100 substeps: 0.1 s of flow as in the headline's 500) and ``adjoint``
(backward / forward time of the differentiable 64-substep rollout of a
99,452-particle block).

Output: one JSON line on rank 0.  ``value`` is timed with CUDA events on the
solver's stream around K substeps whose inputs are already on the GPU; ``e2e``
times the same substeps through the public Python API with the fluid state
copied from pinned host memory before each substep and positions / velocities
and the step scalars copied back after it.  ``roofline`` takes the step phase
with the largest share of the step time, its algorithmic bytes per launch
(each particle's own fields once per sweep: ``ALGO_BYTES_3D``) and its mean
launch time measured here with
CUDA events (``tsph_profile_phases``).  ``cpu_baseline`` times the C
restatement of the reference (``oracle/sph_port.c``, FP32, OpenMP on every host
core) on a bounded number of substeps of the same scene.

Multi-GPU: the single scene does not shard (it has no independent parts), so
N ranks run N independent replicas (weak scaling, no collective in the timed
region); ``value`` sums the replicas.  ``--impl reference`` runs the reference's
CPU algorithm (the C restatement: Taichi, which the reference compiles its
kernels with, is not installed) on rank 0 only.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "particle-steps/s"
UNIT = "particle-steps/s"

# Algorithmic bytes per particle per launch of each phase (FP32, 3D, s = 12 bytes
# per vector): each particle's own fields read or written once; neighbour reads
# are served on chip.  (fluid bytes, boundary bytes)
ALGO_BYTES_3D = {
    "grid": (24, 24),        # pos read, key write/read, slot write
    "density": (24, 16),     # pos, mass -> density, alpha  |  pos, mass
    "psi": (36, 16),         # pos, v_adv, mass, density -> psi_adv  |  pos, mass
    "vel": (48, 16),         # pos, psi_adv, alpha, mass, v_adv r/w  |  pos, mass
    "advect": (44, 0),       # pos, v, mass, density -> v_adv
    "unsort": (52, 0),       # v_adv, pos, mass -> pos, v
    "cfl": (12, 0),
}


# FP32 operations per evaluation in the neighbour sweeps, counted from the CUDA
# source (add / mul 1, FMA 2, rsqrt 1; both spline branches are evaluated):
# a candidate test (dx, r^2) 8; a fluid particle's pair in the density sweep's
# list pass 50 with a fluid neighbour, 44 with a boundary one (it recomputes the
# test); a boundary particle's pair beyond its candidate test 19 with a boundary
# neighbour, 34 with a fluid one; a list pair in psi 32 and in vel 28.
FLOPS = {"cand": 8, "dens_ff": 50, "dens_fb": 44, "dens_bb": 19, "dens_bf": 34, "psi": 32, "vel": 28}


def alu_roofline(solver, ph, top):
    """Secondary (arithmetic) roofline of the neighbour sweeps: FP32 operations
    per launch from the exact pair and candidate counts of the current state,
    over the launch time, against the GPU's FMA rate measured here."""
    from tichi_sph_gb300.sph import fp32_fma_peak
    fc, _, bc, _ = solver.neighbor_stats()
    cf, cb = solver.candidate_stats()
    ff, fb = int(fc[:, 0].sum()), int(fc[:, 1].sum())
    bf, bb = int(bc[:, 0].sum()), int(bc[:, 1].sum())
    cand = int(cf.sum()) + int(cb.sum())
    flops = {
        "density": FLOPS["cand"] * cand + FLOPS["dens_ff"] * ff + FLOPS["dens_fb"] * fb + FLOPS["dens_bb"] * bb
        + FLOPS["dens_bf"] * bf,
        "psi": FLOPS["psi"] * (ff + fb),
        "vel": FLOPS["vel"] * (ff + fb),
    }
    peak = fp32_fma_peak()
    per = {k: flops[k] / (ph[k] * 1e-3) / 1e12 for k in flops}
    k = top if top in flops else max(flops, key=lambda x: ph[x])
    return {"bound": "fp32", "kernel": k, "achieved": per[k], "peak": peak, "unit": "TFLOP/s",
            "frac": per[k] / peak, "peak_source": "measured by bench.py on this GPU (FMA chains, tsph_fp32_fma_peak)",
            "flops_per_launch": flops, "achieved_per_phase": per, "frac_per_phase": {x: per[x] / peak for x in per},
            "pairs_per_step": {"fluid_fluid": ff, "fluid_boundary": fb, "boundary_fluid": bf,
                               "boundary_boundary": bb},
            "density_candidates_per_launch": cand,
            "flops_per_evaluation": FLOPS}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return None, 0, 1
    import torch.distributed as dist
    import torch
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    dist.init_process_group(backend)
    return dist, dist.get_rank(), ws


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id):
        self.gpu_id = gpu_id
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.QUERY, "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", self.gpu_id],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _ncu_traffic(kernel):
    """DRAM bytes per particle of one launch of `kernel`, from the committed ncu
    summary ``profiles/ncu_traffic.txt`` (lines: kernel dram_bytes fluid bound)."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for ln in f:
            t = ln.split()
            if len(t) >= 4 and t[0] == kernel and not ln.startswith("#"):
                return float(t[1]), int(t[2]), int(t[3])
    return None


def build_sim(n_side, device, spacing=0.01):
    from tichi_sph_gb300 import sph_config, workloads
    from tichi_sph_gb300.simulation import Simulation
    cfg_d, scen_d = workloads.dambreak_3d(n_side, spacing)
    cfg = sph_config.Config(cfg_d, scen_d)
    sim = Simulation(cfg, device=device)
    sim.init_scenario()
    return cfg, sim


def cpu_baseline(n_side, budget_s, max_steps, spacing=0.01):
    """C restatement of the reference (FP32, OpenMP) on the same initial state."""
    from oracle.port import PortSim
    from tichi_sph_gb300 import sph_config, workloads
    from tichi_sph_gb300.simulation import Simulation
    cfg_d, scen_d = workloads.dambreak_3d(n_side, spacing)
    cfg = sph_config.Config(cfg_d, scen_d)
    sim = Simulation(cfg, device="cpu")
    sim.init_scenario()
    keys = ["pos", "vel", "volume_frac", "rest_volume", "mass", "rest_density"]
    fa = {k: getattr(sim.fluid, k)[:sim.fluid.part_num[None]].numpy() for k in keys}
    ba = {k: getattr(sim.bound, k)[:sim.bound.part_num[None]].numpy() for k in keys}
    port = PortSim(cfg, fa, ba)
    nf = sim.fluid.part_num[None]
    t0 = time.perf_counter()
    steps = 0
    iters = []
    while steps < max_steps:
        st = port.substep()
        iters.append((st["div_iter"], st["incom_iter"]))
        steps += 1
        if time.perf_counter() - t0 > budget_s:
            break
    el = time.perf_counter() - t0
    thr = port.threads()
    port.close()
    return {"value": nf * steps / el, "unit": UNIT, "cores": thr, "kind": "port",
            "sample": "%d substeps of the full scene from rest (%d fluid + %d boundary particles), %.1f s, "
                      "C restatement of the reference kernels (oracle/sph_port.c), FP32" % (
                          steps, nf, sim.bound.part_num[None], el),
            "ms_per_step": el / steps * 1e3, "iters": iters, "n_bound": sim.bound.part_num[None]}


def run_batched(n_scenes, steps, warmup, dev, dist=None, rank=0, ws=1, hostloop=False):
    """Scenes of workloads.batched_dambreaks stepped (a) as one batch and (b) one at
    a time, each through its own plain context: particle-steps/s of both.  With
    several ranks the scenes are split by partition_scenes (no collective while
    stepping); times are the maximum over ranks, particle counts the totals.
    ``hostloop``: the batch launches every kernel on its own (as profilers list
    them) instead of one CUDA graph per substep."""
    import torch
    from tichi_sph_gb300 import sph_config, workloads, Solver
    from tichi_sph_gb300.batch import BatchSolver, gather_scenes
    from tichi_sph_gb300.partition import partition_scenes, max_over_ranks, gather_scene_stats
    from tichi_sph_gb300.simulation import Simulation
    scenes = workloads.batched_dambreaks(n_scenes)
    counts = [sc["fluid"]["max_part_num"] for _, sc in scenes]
    mine = partition_scenes(counts, ws)[rank]
    sims = []
    for i in mine:
        c, sc = scenes[i]
        cfg = sph_config.Config(c, sc)
        sim = Simulation(cfg, device="cpu")
        sim.init_scenario()
        sims.append(sim)
    fluid, bound, nf, nb = gather_scenes(sims, device=dev)
    batch = BatchSolver([s.config for s in sims], fluid, bound, nf, nb, use_graph=not hostloop)
    stream = torch.cuda.current_stream(dev)
    for _ in range(warmup):
        batch.substep()
    torch.cuda.synchronize(dev)
    s0 = batch.stats()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        batch.substep()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    ms = max_over_ranks(e0.elapsed_time(e1) / steps, dist)
    s1 = batch.stats()
    batch.close()
    per_scene = [(b["total_div_iter"] - a["total_div_iter"], b["total_incom_iter"] - a["total_incom_iter"])
                 for a, b in zip(s0, s1)]
    all_scenes = gather_scene_stats(per_scene, mine, n_scenes, dist)
    if all_scenes is not None:
        kd = sum(x[0] for x in all_scenes) / (steps * n_scenes)
        ki = sum(x[1] for x in all_scenes) / (steps * n_scenes)
    else:
        kd = ki = None
    solos = [Solver(s.config, s.fluid, s.bound) for s in sims]
    for _ in range(warmup):
        for so in solos:
            so.substep()
    torch.cuda.synchronize(dev)
    e0.record(stream)
    for _ in range(steps):
        for so in solos:
            so.substep()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    ms_seq = max_over_ranks(e0.elapsed_time(e1) / steps, dist)
    for so in solos:
        so.close()
    tot = sum(counts)
    return {"n_scenes": n_scenes, "fluid_particles": tot, "boundary_particles": _sum_over_ranks(sum(nb), dist),
            "scenes_per_rank": len(mine),
            "value": tot / (ms / 1e3), "sequential_value": tot / (ms_seq / 1e3), "speedup": ms_seq / ms,
            "ms_per_step": ms, "sequential_ms_per_step": ms_seq, "mean_div_iter": kd, "mean_incom_iter": ki,
            "steps": steps, "warmup": warmup}


def _sum_over_ranks(v, dist):
    if dist is None:
        return int(v)
    import torch
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([int(v)], dtype=torch.int64, device=dev)
    dist.all_reduce(t)
    return int(t.item())


def batched_line(res, args, ws):
    return {"metric": "particle-steps/s, batched vs plain", "value": res["value"], "unit": UNIT,
            "n_gpus": ws, "steps": res["steps"], "warmup": res["warmup"], "ms_per_step": res["ms_per_step"],
            "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "%d independent 3D dam breaks (seed 4), fluid log-uniform in [2k, 200k], aspect "
                                   "[0.5, 2], rest density [800, 1200], spacing 0.01" % res["n_scenes"],
                       "parallelism": "scenes split across %d rank(s), greedy balance on fluid counts, no collective "
                                      "while stepping" % ws,
                       "fluid_particles": res["fluid_particles"], "boundary_particles": res["boundary_particles"],
                       "sequential_value": res["sequential_value"], "speedup_vs_sequential": res["speedup"],
                       "sequential_ms_per_step": res["sequential_ms_per_step"],
                       "mean_div_iter": res["mean_div_iter"], "mean_incom_iter": res["mean_incom_iter"]}}


def run_other(kind, steps, warmup, dev, develop=0, n_side=100, hostloop=False):
    """The two-phase VFSPH block pair (two cubes of ``n_side``^3 particles), the
    2D dam break, or (``dambreak3d_cs10``) the headline dam break at a five times
    larger time step (solver_cs 10, dt up to 1e-3), where the Jacobi solves
    iterate past their floor, through the plain path: ``develop`` untimed
    substeps from rest, ``warmup`` more, then ``steps`` timed; ``hostloop``: the
    warm-up and timed substeps launch every kernel on its own."""
    import numpy as np
    import torch
    from tichi_sph_gb300 import sph_config, workloads
    from tichi_sph_gb300.simulation import Simulation
    if kind == "twophase3d":
        c, sc, noise = workloads.twophase_3d(n_side=n_side)
        fbm = True
    elif kind == "dambreak3d_cs10":
        c, sc = workloads.dambreak_3d(n_side)
        c["solver_cs"] = 10
        noise, fbm = None, False
    else:
        c, sc = workloads.dambreak_2d()
        noise, fbm = None, False
    cfg = sph_config.Config(c, sc)
    sim = Simulation(cfg, device=dev, fbm=fbm)
    sim.init_scenario()
    nf = sim.fluid.part_num[None]
    if noise is not None:
        vf = noise(sim.fluid.volume_frac[:nf].cpu().numpy())
        sim.fluid.volume_frac[:nf] = torch.as_tensor(vf, device=dev)
        sim.fluid.update_mass_all()
    s = sim.solver
    stream = torch.cuda.current_stream(dev)
    for _ in range(develop):
        s.substep()
    if hostloop:
        s.set_graph_mode(False)
    for _ in range(warmup):
        s.substep()
    torch.cuda.synchronize(dev)
    s0 = s.stats()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        s.substep()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / steps
    s1 = s.stats()
    vf = sim.fluid.volume_frac[:nf].cpu().numpy().astype(np.float64)
    s.close()
    return {"kind": kind, "fluid_particles": nf, "boundary_particles": sim.bound.part_num[None], "ms": ms,
            "steps": steps, "warmup": warmup, "develop": develop,
            "div": (s1["total_div_iter"] - s0["total_div_iter"]) / steps,
            "inc": (s1["total_incom_iter"] - s0["total_incom_iter"]) / steps,
            "fbm": (s1["total_fbm_passes"] - s0["total_fbm_passes"]) / steps,
            "max_comp": s1["max_dens_compression"], "vf_sum_err": float(np.abs(vf.sum(axis=1) - 1).max()),
            "vf_min": float(vf.min())}


def other_line(res, args, ws):
    n3 = res["fluid_particles"] // 2
    side = "%.2f m cubes" % (round(n3 ** (1 / 3)) * 0.01)
    desc = {"twophase3d": "3D two-phase VFSPH, two %s (rest density 1000 / 500) of %d particles each, "
                          "spacing 0.01, surface tension 0.07, volume-fraction update on" % (side, n3),
            "dambreak2d": "2D DFSPH dam break, 1.0 x 2.0 m block at 0.02 m (5,000 particles), 4 x 4 m box, "
                          "dt 1e-3",
            "dambreak3d_cs10": "3D DFSPH dam break, %d fluid + %d boundary particles, h=0.02, solver_cs 10 "
                               "(dt<=1e-3, CFL), rho tol 0.1%%, div tol 1%%" % (res["fluid_particles"],
                                                                              res["boundary_particles"])}[res["kind"]]
    return {"metric": METRIC, "value": res["fluid_particles"] * ws / (res["ms"] / 1e3), "unit": UNIT, "n_gpus": ws,
            "steps": res["steps"], "warmup": res["warmup"], "ms_per_step": res["ms"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": desc, "fluid_particles": res["fluid_particles"],
                       "boundary_particles": res["boundary_particles"], "mean_div_iter": res["div"],
                       "mean_incom_iter": res["inc"], "mean_fbm_passes": res["fbm"],
                       "max_density_error": res["max_comp"], "max_abs_volume_fraction_sum_error": res["vf_sum_err"],
                       "min_volume_fraction": res["vf_min"]}}


def extra_workloads(dev, args):
    """The other configurations of the hot path at N = 1, for the headline line:
    the two-phase VFSPH pair (end of its 300-substep run), the 2D dam break
    (substeps 4..1,000 of its run), the headline dam break at solver_cs 10 (its
    solves iterate) and the adjoint's backward / forward ratio."""
    out = {}
    tp = run_other("twophase3d", 20, 3, dev, develop=277)
    out["twophase3d"] = {"value": tp["fluid_particles"] / (tp["ms"] / 1e3), "unit": UNIT, "ms_per_step": tp["ms"],
                         "window": "substeps %d..%d of a 300-substep run from rest" % (
                             tp["develop"] + tp["warmup"] + 1, tp["develop"] + tp["warmup"] + tp["steps"]),
                         "workload": other_line(tp, args, 1)["config"]["workload"],
                         **{k: other_line(tp, args, 1)["config"][k] for k in (
                             "fluid_particles", "boundary_particles", "mean_div_iter", "mean_incom_iter",
                             "mean_fbm_passes", "max_density_error", "max_abs_volume_fraction_sum_error")}}
    d2 = run_other("dambreak2d", 997, 3, dev)
    out["dambreak2d"] = {"value": d2["fluid_particles"] / (d2["ms"] / 1e3), "unit": UNIT, "ms_per_step": d2["ms"],
                         "window": "substeps 4..1000 of the 1,000-substep run from rest",
                         "workload": other_line(d2, args, 1)["config"]["workload"],
                         **{k: other_line(d2, args, 1)["config"][k] for k in (
                             "fluid_particles", "boundary_particles", "mean_div_iter", "mean_incom_iter",
                             "max_density_error")}}
    it = run_other("dambreak3d_cs10", 20, 3, dev, develop=77)
    out["dambreak3d_cs10"] = {"value": it["fluid_particles"] / (it["ms"] / 1e3), "unit": UNIT, "ms_per_step": it["ms"],
                              "window": "substeps %d..%d of a 100-substep run from rest (0.1 s of flow, the time the "
                                        "headline's 500 substeps cover)" % (
                                            it["develop"] + it["warmup"] + 1, it["develop"] + it["warmup"] + it["steps"]),
                              "workload": other_line(it, args, 1)["config"]["workload"],
                              **{k: other_line(it, args, 1)["config"][k] for k in (
                                  "fluid_particles", "boundary_particles", "mean_div_iter", "mean_incom_iter",
                                  "max_density_error")}}
    ad = run_adjoint(3, 1, dev)
    al = adjoint_line(ad, args, 1)
    out["adjoint"] = {"metric": "backward/forward time", "value": ad["ratio"], "unit": "ratio",
                      "higher_is_better": False, "reps": ad["reps"], **al["config"]}
    return out


def run_adjoint(reps, warmup, dev, substeps=64, checkpoint_every=8, gamma=0.0):
    """Config of the differentiable form: a 99,452-particle block, 64 substeps at
    dt 5e-4, loss = |centre of mass - target|^2 + 0.1 mean density error^2,
    gradients with respect to the initial velocities and the viscosity.  Times
    the forward (rollout + final density) and the backward (recompute of every
    checkpoint segment but the last + the reverse sweeps) with CUDA events.
    ``gamma`` != 0 adds surface tension (forward and reverse)."""
    import torch
    from tichi_sph_gb300 import sph_config, workloads
    from tichi_sph_gb300.adjoint import DiffRollout, com_density_loss
    from tichi_sph_gb300.simulation import Simulation
    c, sc_, vel, target = workloads.diff_block(gamma=gamma)
    cfg = sph_config.Config(c, sc_)
    sim = Simulation(cfg, device=dev)
    sim.init_scenario()
    n = sim.fluid.part_num[None]
    roll = DiffRollout(cfg, sim.fluid, sim.bound, substeps, checkpoint_every=checkpoint_every)
    v0 = torch.as_tensor(vel(n), device=dev)
    tgt = torch.as_tensor(target, device=dev)
    mass = sim.fluid.mass[:n].double()
    rho0 = sim.fluid.rest_density[:n].double()
    stream = torch.cuda.current_stream(dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    fw, bw, gnorm, gmu, loss = [], [], 0.0, 0.0, 0.0
    for r in range(warmup + reps):
        v = v0.clone().requires_grad_(True)
        mu = torch.tensor(0.01, dtype=torch.float64, requires_grad=True)
        torch.cuda.synchronize(dev)
        ev[0].record(stream)
        x, _, rho = roll(v, mu)
        L = com_density_loss(x.double(), rho.double(), mass, rho0, tgt)
        ev[1].record(stream)
        L.backward()
        ev[2].record(stream)
        torch.cuda.synchronize(dev)
        if r >= warmup:
            fw.append(ev[0].elapsed_time(ev[1]))
            bw.append(ev[1].elapsed_time(ev[2]))
        gnorm, gmu, loss = float(v.grad.norm()), float(mu.grad), float(L.detach())
    st = roll.solver.stats()
    roll.close()
    fwm, bwm = sum(fw) / len(fw), sum(bw) / len(bw)
    return {"n": n, "nb": sim.bound.part_num[None], "substeps": substeps, "checkpoint_every": checkpoint_every,
            "forward_ms": fwm, "backward_ms": bwm, "ratio": bwm / fwm, "grad_v_norm": gnorm, "grad_mu": gmu,
            "loss": loss, "reps": reps, "warmup": warmup, "last_div_iter": st["div_iter"],
            "last_incom_iter": st["incom_iter"], "gamma": gamma}


def adjoint_line(res, args, ws):
    return {"metric": "backward/forward time", "value": res["ratio"], "unit": "ratio", "n_gpus": ws,
            "steps": res["reps"], "warmup": res["warmup"], "ms_per_step": res["forward_ms"] + res["backward_ms"],
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "differentiable DFSPH: %d-particle block (46 x 46 x 47 at 0.01 m) in a 3-layer "
                                   "tank (%d boundary), %d substeps at dt 5e-4, checkpoint every %d; loss |CoM - "
                                   "target|^2 + 0.1 mean((rho - rho0) / rho0)^2; d/d(initial velocities), d/d(mu)%s"
                                   % (res["n"], res["nb"], res["substeps"], res["checkpoint_every"],
                                      "; surface tension %g" % res["gamma"] if res["gamma"] else ""),
                       "forward_ms": res["forward_ms"], "backward_ms": res["backward_ms"],
                       "forward_particle_steps_per_s": res["n"] * res["substeps"] / (res["forward_ms"] / 1e3),
                       "loss": res["loss"], "grad_v_norm": res["grad_v_norm"], "grad_mu": res["grad_mu"],
                       "last_div_iter": res["last_div_iter"], "last_incom_iter": res["last_incom_iter"]}}


def run_reference(args, rank, ws):
    if rank != 0:
        return 0
    n_side = args.n_side
    res = cpu_baseline(n_side, budget_s=args.ref_budget, max_steps=args.warmup + args.steps, spacing=args.spacing)
    nf = n_side ** 3
    line = {
        "metric": METRIC, "value": res["value"], "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
        "steps": len(res["iters"]), "warmup": 0, "ms_per_step": res["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "3D DFSPH dam break, %d fluid + %d boundary particles, h=%g, dt<=%g (CFL), "
                               "rho tol 0.1%%, div tol 1%%" % (nf, res["n_bound"], 2 * args.spacing, args.spacing / 50),
                   "window": "substeps 1..%d of the run from rest (a bounded CPU sample; the GPU arm times the "
                             "end of the 500-substep run, the developed flow; both at the solvers' floor of two "
                             "iterations each)" % len(res["iters"]),
                   "fluid_particles": nf},
        "cpu_baseline": {k: res[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": res["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "Taichi (the reference's kernel compiler) is not installed; the reference's kernel sequence "
                "runs as its C restatement on the host cores",
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--develop", type=int, default=-1,
                    help="untimed substeps before the warm-up (-1: 500 - warmup - steps, so the timed window "
                         "ends the 500-substep run)")
    ap.add_argument("--run-length", type=int, default=500, help="substeps of the headline run (for --develop -1)")
    ap.add_argument("--no-extra", action="store_true", help="skip the two-phase, 2D and adjoint workloads")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n-side", type=int, default=100)
    ap.add_argument("--gamma", type=float, default=0.0,
                    help="surface-tension coefficient of the adjoint workload (0: none)")
    ap.add_argument("--spacing", type=float, default=0.01,
                    help="particle spacing of the 3D dam break (the cube is n-side particles wide, the tank fixed)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--ref-budget", type=float, default=150.0)
    ap.add_argument("--hostloop", action="store_true",
                    help="host-driven solver loops instead of the CUDA graph for the warm-up and timed substeps "
                         "(kernels launched one by one, as profilers list them)")
    ap.add_argument("--no-profile", action="store_true", help="skip the per-phase timing (roofline)")
    ap.add_argument("--tpp", type=int, default=0, help="threads per particle (0: autotune after warm-up)")
    ap.add_argument("--workload", default="dambreak3d",
                    choices=["dambreak3d", "batched", "twophase3d", "dambreak2d", "dambreak3d_cs10", "adjoint"],
                    help="dambreak3d: the headline line; the others print their own line")
    ap.add_argument("--batch-scenes", type=int, default=256,
                    help="scenes of the batched measurement added to the headline line (0: skip)")
    ap.add_argument("--batch-steps", type=int, default=10)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    dist, rank, ws = _dist()
    if args.impl == "reference":
        rc = run_reference(args, rank, ws)
        if dist:
            dist.destroy_process_group()
        return rc

    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if args.workload == "batched":
        res = run_batched(256, args.steps, args.warmup, dev, dist, rank, ws, hostloop=args.hostloop)
        if rank == 0:
            print(json.dumps(batched_line(res, args, ws)), flush=True)
        if dist:
            dist.destroy_process_group()
        return 0
    if args.workload == "adjoint":
        res = run_adjoint(args.steps, args.warmup, dev, gamma=args.gamma)
        if rank == 0:
            print(json.dumps(adjoint_line(res, args, ws)), flush=True)
        if dist:
            dist.destroy_process_group()
        return 0
    if args.workload in ("twophase3d", "dambreak2d", "dambreak3d_cs10"):
        res = run_other(args.workload, args.steps, args.warmup, dev, develop=max(args.develop, 0),
                        n_side=args.n_side, hostloop=args.hostloop)
        if rank == 0:
            print(json.dumps(other_line(res, args, ws)), flush=True)
        if dist:
            dist.destroy_process_group()
        return 0
    cfg, sim = build_sim(args.n_side, dev, args.spacing)
    solver = sim.solver
    nf, nb = sim.fluid.part_num[None], sim.bound.part_num[None]
    stream = torch.cuda.current_stream(dev)

    tune = None
    if args.tpp:
        solver.set_threads_per_particle(args.tpp)
    develop = args.develop if args.develop >= 0 else max(0, args.run_length - args.warmup - args.steps)
    for _ in range(develop):
        solver.substep()
    if args.hostloop:
        # the warm-up and timed substeps launch every kernel on its own (the
        # development above runs as graphs)
        solver.set_graph_mode(False)
    for i in range(args.warmup):
        solver.substep()
        if i == 0 and not args.tpp:
            tune = solver.autotune()
    torch.cuda.synchronize(dev)
    s0 = solver.stats()

    def barrier():
        if dist:
            dist.barrier()

    uuid = None
    try:
        uuid = "GPU-" + str(torch.cuda.get_device_properties(dev).uuid)
    except Exception:
        uuid = str(local)
    clocks = ClockSampler(uuid)
    clocks.start()
    barrier()
    torch.cuda.synchronize(dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        solver.substep()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    barrier()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    s1 = solver.stats()
    if dist:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_step = ms / args.steps
    value = nf * args.steps * ws / (ms / 1e3)
    k_div = (s1["total_div_iter"] - s0["total_div_iter"]) / args.steps
    k_inc = (s1["total_incom_iter"] - s0["total_incom_iter"]) / args.steps
    launches = int(args.steps * s1["launches_per_step"] + s1["launches_per_iter"] *
                   ((s1["total_div_iter"] - s0["total_div_iter"]) + (s1["total_incom_iter"] - s0["total_incom_iter"])))

    # per-phase launch times (CUDA events on the solver's stream), for the roofline
    if args.no_profile:
        ph = {k: 1.0 for k in ("cfl", "grid", "density", "psi", "vel", "advect", "unsort")}
    else:
        ph = solver.profile_phases(reps=5)
    # the divergence solve's first psi sweep runs inside the density launch
    per_step = {"cfl": 1, "grid": 1, "density": 1, "psi": max(k_div - 1.0, 0.0) + k_inc, "vel": k_div + k_inc,
                "advect": 1, "unsort": 1}
    share = {k: ph[k] * per_step[k] for k in ph}
    top = max(share, key=share.get)
    fb, bb = ALGO_BYTES_3D[top]
    algo_bytes = fb * nf + bb * nb
    achieved = algo_bytes / (ph[top] / 1e3) / 1e9
    peak, peak_kind = _peaks()
    tr = _ncu_traffic(top)
    traffic = None
    if tr is not None:
        dram, f0, b0 = tr
        traffic = dram * (fb * nf + bb * nb) / max(fb * f0 + bb * b0, 1)
    roofline = {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)"
                if peak_kind == "measured" else "fallback 6.8 TB/s",
                "algorithmic_bytes_per_launch": algo_bytes, "launch_ms": ph[top],
                "phase_ms_per_launch": ph, "phase_share_of_step": {k: share[k] / sum(share.values()) for k in share}}

    alu = None
    if not args.no_profile:
        alu = alu_roofline(solver, ph, top)

    # end to end through the public API with host buffers
    e2e = None
    if not args.no_e2e:
        keys = ["pos", "vel", "mass", "rest_density", "rest_volume", "volume_frac"]
        # the fluid state lives in pinned host memory and round-trips every substep
        host_in = {k: getattr(sim.fluid, k)[:nf].detach().to("cpu").pin_memory() for k in keys}
        host_out = {k: host_in[k] for k in ("pos", "vel")}
        h2d = sum(t.numel() * t.element_size() for t in host_in.values())
        d2h = sum(t.numel() * t.element_size() for t in host_out.values()) + 8 * 5
        barrier()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        e2 = torch.cuda.Event(enable_timing=True)
        e3 = torch.cuda.Event(enable_timing=True)
        e2.record(stream)
        for _ in range(args.steps):
            for k, t in host_in.items():
                getattr(sim.fluid, k)[:nf].copy_(t, non_blocking=True)
            solver.substep()
            for k, t in host_out.items():
                t.copy_(getattr(sim.fluid, k)[:nf], non_blocking=True)
            solver.stats()  # the step's scalars to the host (synchronises)
        e3.record(stream)
        torch.cuda.synchronize(dev)
        wall = time.perf_counter() - t0
        barrier()
        ems = e2.elapsed_time(e3)
        if dist:
            t = torch.tensor([ems], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ems = float(t.item())
        e2e = {"value": nf * args.steps * ws / (ems / 1e3), "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": ems / args.steps, "host_wall_s": wall}

    batched = None
    if args.batch_scenes > 0:
        solver.close()
        b = run_batched(args.batch_scenes, args.batch_steps, 3, dev, dist, rank, ws)
        batched = {k: b[k] for k in ("n_scenes", "fluid_particles", "boundary_particles", "value", "sequential_value",
                                     "speedup", "ms_per_step", "sequential_ms_per_step", "mean_div_iter",
                                     "mean_incom_iter")}
        batched["unit"] = UNIT
        batched["workload"] = ("%d independent 3D dam breaks, fluid counts log-uniform in [2k, 200k] (seed 4), "
                               "batched in one launch vs stepped one at a time through the plain path" % b["n_scenes"])

    extra = {}
    if ws == 1 and not args.no_extra:
        solver.close()
        extra = extra_workloads(dev, args)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cb = cpu_baseline(args.n_side, budget_s=args.cpu_budget, max_steps=20, spacing=args.spacing)
        cpu = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "3D DFSPH dam break, %d fluid + %d boundary particles, h=%g, dt<=%g (CFL), "
                                   "rho tol 0.1%%, div tol 1%%" % (nf, nb, 2 * args.spacing, args.spacing / 50),
                       "window": "substeps %d..%d of the run from rest (%d untimed to develop the flow, %d warm-up)" % (
                           develop + args.warmup + 1, develop + args.warmup + args.steps, develop, args.warmup),
                       "fluid_particles": nf, "boundary_particles": nb, "parallelism": "replicas" if ws > 1 else "single",
                       "mean_div_iter": k_div, "mean_incom_iter": k_inc,
                       "density_error_after_window": s1["compression"],
                       "max_density_error": s1["max_dens_compression"],
                       "l2": "inputs larger than L2 (per-step state ~%d MB > 129 MB)" % round(400 * nf / 1e6),
                       "threads_per_particle": solver.tpp, "autotune_ms": tune,
                       "graph": "host-driven solver loops" if args.hostloop else
                       "one CUDA graph per substep, device-side while nodes"},
            "roofline": roofline,
            "alu_roofline": alu,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": launches,
            "clocks": clk,
            "batched": batched,
        }
        line.update(extra)
        print(json.dumps(line), flush=True)
    if solver.ctx:
        solver.close()
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
