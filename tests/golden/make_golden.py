"""Generate golden vectors by running the Tichi_SPH reference's own kernels.

Test infrastructure, run by hand where the reference source is present
(``TICHI_REFERENCE=<Tichi_SPH tree> python tests/golden/make_golden.py [scene ...]``);
the fixtures it writes are committed and the tests never need the reference at
run time.

Taichi is not installed here, so the reference modules are imported on top of the
pure-Python Taichi stand-in in ``tests/golden/taichi_shim`` and every kernel body of
``sph.py`` / ``sph_obj.py`` / ``sph_util.py`` / ``sph_config.py`` runs as written.
The reference's ``main.py`` cannot be imported (it opens a GGUI window at import,
``main.py:383-415``), so ``_substep`` below replays its per-substep sequence:
``run_step`` (``main.py:339-352``) and ``sph_step`` (``main.py:175-256``), with the
volume-fraction (FBM) block ``main.py:244-250`` enabled for VFSPH scenes, and --
for the ``wcsph*`` scenes -- the weakly compressible pressure block
``main.py:238-242`` and the particle-to-grid map ``main.py:254`` (both shipped
commented out) enabled; ``map_velocity`` runs on a ``Grid`` whose shape is
ceil((rt - lb) / dist) per axis, the intent of ``sph_obj.py:326`` (whose
expression divides only ``lb``).

For each scene in ``tests/golden/scenes`` two child processes run:

1. ``TAICHI_SHIM_FP=f32``: the reference's emitters (``scene_add_cube`` /
   ``scene_add_box``, ``sph_obj.py:102-180``) build the initial state with f32
   field stores, exactly as Taichi's ``default_fp=f32`` would; VFSPH scenes then get
   seeded per-particle volume-fraction noise and the reference's ``SPH_update_mass``.
   Saved as ``<scene>.init.npz``.
2. ``TAICHI_SHIM_FP=f64``: the same objects, loaded with that initial state, are
   stepped ``STEPS[scene]`` substeps with f64 field storage; every field and
   counter after each substep is saved as ``<scene>.steps.npz``.  f64 storage makes
   these the reference algorithm's values without f32 rounding, which is what the
   FP64 oracle is pinned against.
"""
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("TICHI_REFERENCE", "")
SCENES = os.path.join(HERE, "scenes")
STEPS = {"dfsph2d": 3, "dfsph2d_r2": 2, "dfsph3d": 2, "vfsph2d": 3, "vfsph3d": 2, "edge2d": 2,
         "wcsph2d": 3, "wcsph3d": 2, "inlet3d": 8}
# scenes whose scenario emits at run time (an inlet, objects with a "time"):
# each substep starts with the reference's refresh_scenario (main.py:346)
EMIT_SCENES = {"inlet3d"}
FBM_SCENES = {"vfsph2d", "vfsph3d"}
WC_SCENES = {"wcsph2d", "wcsph3d"}
VF_NOISE_SEED = 3

PARTICLE_FIELDS = [
    "pos", "vel", "vel_adv", "acce", "acce_adv", "mass", "rest_density", "rest_volume",
    "volume_frac", "volume_frac_tmp", "W", "sph_density", "sph_compression", "psi_adv",
    "alpha", "alpha_1", "alpha_2", "normal", "drift_vel", "fbm_zeta", "flag",
    "neighb_cell_seq", "neighb_cell_structured_seq", "pressure", "pressure_force", "W_grad",
]
STATE_IN = ["pos", "vel", "volume_frac", "rest_volume", "mass", "rest_density"]


def _child(scene, mode):
    if not REF or not os.path.isdir(REF):
        raise SystemExit("set TICHI_REFERENCE to the Tichi_SPH source tree (the folder holding sph.py)")
    sys.dont_write_bytecode = True
    sys.path.insert(0, os.path.join(HERE, "taichi_shim"))
    sys.path.insert(0, REF)
    sys.argv = ["main.py", "-c", os.path.join(SCENES, scene + ".config.json"),
                "-s", os.path.join(SCENES, scene + ".scenario.json")]
    import sph  # noqa: E402  (runs sph_config at import, sph_config.py:27-235)
    R = sph
    config = R.config
    # main.py:8-12 without the Eulerian Grid (unused; it would allocate 328^3 cells)
    ngrid = R.Ngrid()
    fluid = R.Fluid(max_part_num=config.fluid_max_part_num[None])
    bound = R.Fluid(max_part_num=config.bound_max_part_num[None])
    objs = {"fluid": fluid, "bound": bound}
    gv = R.GlobalVariable()
    scenario = _Scenario(R, config, objs, gv)
    scenario.init_scenario()

    if mode == "f32":
        if scene in FBM_SCENES:
            # seeded +-0.05 noise on the volume fractions, clipped and renormalised
            rng = np.random.default_rng(VF_NOISE_SEED)
            n = fluid.part_num[None]
            vf = fluid.volume_frac.to_numpy()
            noisy = np.clip(vf[:n] + rng.uniform(-0.05, 0.05, vf[:n].shape), 0.0, 1.0)
            noisy /= noisy.sum(axis=1, keepdims=True)
            vf[:n] = noisy.astype(np.float32)
            fluid.volume_frac.from_numpy(vf)
            R.SPH_update_mass(fluid)
        out = {"solver_type": R.solver_type}
        for name, obj in objs.items():
            n = obj.part_num[None]
            out[name + "_n"] = n
            for f in STATE_IN:
                out[name + "_" + f] = getattr(obj, f).to_numpy()[:n]
        np.savez_compressed(os.path.join(HERE, scene + ".init.npz"), **out)
        return

    init = np.load(os.path.join(HERE, scene + ".init.npz"))
    for name, obj in objs.items():
        n = int(init[name + "_n"])
        assert obj.part_num[None] == n, (name, obj.part_num[None], n)
        for f in STATE_IN:
            arr = getattr(obj, f).to_numpy()
            arr[:n] = init[name + "_" + f]
            getattr(obj, f).from_numpy(arr)

    fbm = scene in FBM_SCENES
    wc = scene in WC_SCENES
    grid = _Grid(R, config) if wc else None
    rec = {}
    if grid is not None:
        rec["grid_lb"], rec["grid_dist"], rec["grid_shape"] = grid.lb, grid.dist, np.array(grid.shape)
    for step in range(STEPS[scene]):
        if scene in EMIT_SCENES:
            scenario.refresh_scenario()
        _substep(R, config, ngrid, fluid, bound, gv, fbm, wc, grid)
        p = "s%d_" % step
        if grid is not None:
            rec[p + "grid_vel"] = grid.vel.to_numpy()
        rec[p + "dt"] = config.dt[None]
        rec[p + "time_count"] = gv.time_count
        rec[p + "div_iter"] = gv.div_iter_count
        rec[p + "incom_iter"] = gv.incom_iter_count
        rec[p + "compression"] = fluid.compression[None]
        rec[p + "kinetic_energy"] = fluid.statistics_kinetic_energy[None]
        rec[p + "potential_energy"] = fluid.statistics_gravity_potential_energy[None]
        rec[p + "general_flag"] = fluid.general_flag[None]
        for name, obj in objs.items():
            n = obj.part_num[None]
            for f in PARTICLE_FIELDS:
                rec[p + name + "_" + f] = getattr(obj, f).to_numpy()[:n]
        print("  %s step %d: dt=%.6g div=%d incom=%d compression=%.6g" % (
            scene, step, config.dt[None], gv.div_iter_count, gv.incom_iter_count,
            fluid.compression[None]), flush=True)
    np.savez_compressed(os.path.join(HERE, scene + ".steps.npz"), **rec)


class _Scenario:
    """The reference's scenario system, main.py:16-112, replayed on the reference's
    own emitters (``scene_add_cube`` / ``scene_add_box`` / ``scene_add_from_inlet``,
    sph_obj.py:102-163): ``main.py`` cannot be imported (it opens a window), so its
    host-side scheduling is restated here line for line."""

    def __init__(self, R, config, objs, gv):
        self.R, self.config, self.objs, self.gv = R, config, objs, gv
        self.wait = []     # scenario_wait_buffer, main.py:13
        self.inlets = []   # main.py:14

    def inlet_helper_get_dt(self, norm, speed, relaxing_factor):
        """main.py:26-39."""
        norm = np.array(norm) / np.linalg.norm(np.array(norm))
        if speed < 0:
            norm, speed = -norm, -speed
        acc = np.dot(norm, self.config.gravity.to_numpy())
        r = self.config.part_size[1]
        if acc < 1e-6:
            return r * relaxing_factor / speed if speed > 0 else float("inf")
        return ((speed ** 2 + 2 * acc * r) ** 0.5 - speed) / acc * relaxing_factor

    def add_to_scenario(self, part, param):
        """main.py:42-60 (cube, box, inlet)."""
        obj = self.objs[part]
        t = param["type"]
        if t == "cube":
            obj.scene_add_cube(param["start_pos"], param["end_pos"], param["volume_frac"], param["vel"],
                               int(param["color"], 16), param["particle_relaxing_factor"])
        elif t == "box":
            obj.scene_add_box(param["start_pos"], param["end_pos"], param["layers"], param["volume_frac"],
                              param["vel"], int(param["color"], 16), param["particle_relaxing_factor"])
        elif t == "inlet":
            param["obj"] = part
            param["dt"] = self.inlet_helper_get_dt(param["norm"], param["speed"], param["particle_relaxing_factor"])
            param["t_pre"] = self.gv.time_count - param["dt"]
            self.inlets.append(param)
        else:
            raise RuntimeError("golden scenes use cube, box and inlet objects")

    def init_scenario(self):
        """main.py:62-74."""
        for part in self.R.scenario_buffer:
            if part == "sim_env":
                continue
            for param in self.R.scenario_buffer[part]["objs"]:
                if "time" not in param or param["time"] <= 0.0:
                    self.add_to_scenario(part, param)
                else:
                    param["_part"] = part
                    self.wait.append(param)

    def refresh_scenario(self):
        """main.py:81-112 (refresh_inlets after the delayed objects)."""
        gv = self.gv
        for i in range(len(self.wait) - 1, -1, -1):
            param = self.wait[i]
            if param["time"] <= gv.time_count:
                self.add_to_scenario(param["_part"], param)
                self.wait.pop(i)
        for i in range(len(self.inlets) - 1, -1, -1):
            inlet = self.inlets[i]
            if "end_time" in inlet and gv.time_count >= inlet["end_time"]:
                self.inlets.pop(i)
            elif gv.time_count >= inlet["t_pre"] + inlet["dt"]:
                inlet["t_pre"] = gv.time_count
                self.objs[inlet["obj"]].scene_add_from_inlet(
                    inlet["center"], inlet["size"], inlet["norm"], inlet["speed"], inlet["volume_frac"],
                    int(inlet["color"], 16), inlet["particle_relaxing_factor"])


class _Grid:
    """``Grid`` (sph_obj.py:326-344) with the shape ceil((rt - lb) / dist)."""

    def __init__(self, R, config):
        dim = config.dim[None]
        self.lb = config.sim_space_lb[None].to_numpy().astype(np.float64)
        rt = config.sim_space_rt[None].to_numpy().astype(np.float64)
        self.dist = float(config.part_size[1] * config.neighb_grid_size_TO_global_part_size[None])
        self.shape = tuple(int(x) for x in np.ceil((rt - self.lb) / self.dist))
        self.vel = R.ti.Vector.field(dim, float, shape=self.shape)
        self.pos = R.ti.Vector.field(dim, float, shape=self.shape)
        idx = np.stack(np.meshgrid(*[np.arange(n) for n in self.shape], indexing="ij"), -1)
        self.pos.from_numpy(self.lb + idx * self.dist)   # init_pos, sph_obj.py:341-344


def _substep(R, config, ngrid, fluid, bound, gv, fbm, wc=False, grid=None):
    """run_step's substep body (main.py:347-352) around sph_step (main.py:175-256)."""
    R.cfl_condition(fluid)
    gv.time_count += config.dt[None]
    # sph_step
    ngrid.clear_node()
    ngrid.encode(fluid)
    ngrid.encode(bound)
    ngrid.mem_shift()
    ngrid.fill_node(fluid)
    ngrid.fill_node(bound)
    R.SPH_clean_value(fluid)
    R.SPH_clean_value(bound)
    R.SPH_prepare_attr(ngrid, fluid, fluid)
    R.SPH_prepare_attr(ngrid, fluid, bound)
    R.SPH_prepare_attr(ngrid, bound, bound)
    R.SPH_prepare_attr(ngrid, bound, fluid)
    R.SPH_prepare_alpha_1(ngrid, fluid, fluid)
    R.SPH_prepare_alpha_1(ngrid, fluid, bound)
    R.SPH_prepare_alpha_2(ngrid, fluid, fluid)
    R.SPH_prepare_alpha_2(ngrid, bound, fluid)
    R.SPH_prepare_alpha(fluid)
    R.SPH_prepare_alpha(bound)
    gv.div_iter_count = 0
    R.SPH_vel_2_vel_adv(fluid)
    while gv.div_iter_count < config.iter_threshold_min[None] or \
            fluid.compression[None] > config.divergence_threshold[None]:
        R.IPPE_adv_psi_init(fluid)
        R.IPPE_adv_psi(ngrid, fluid, fluid)
        R.IPPE_adv_psi(ngrid, fluid, bound)
        R.IPPE_psi_adv_non_negative(fluid)
        R.IPPE_update_vel_adv(ngrid, fluid, fluid)
        R.IPPE_update_vel_adv(ngrid, fluid, bound)
        gv.div_iter_count += 1
        if gv.div_iter_count > config.iter_threshold_max[None]:
            break
    R.SPH_vel_adv_2_vel(fluid)
    R.SPH_advection_gravity_acc(fluid)
    R.SPH_advection_viscosity_acc(ngrid, fluid, fluid)
    R.SPH_advection_surface_tension_acc(ngrid, fluid, fluid)
    R.SPH_advection_update_vel_adv(fluid)
    gv.incom_iter_count = 0
    while gv.incom_iter_count < config.iter_threshold_min[None] or \
            fluid.compression[None] > config.compression_threshold[None]:
        R.IPPE_adv_psi_init(fluid)
        R.IPPE_adv_psi(ngrid, fluid, fluid)
        R.IPPE_adv_psi(ngrid, fluid, bound)
        R.IPPE_psi_adv_non_negative(fluid)
        R.IPPE_update_vel_adv(ngrid, fluid, fluid)
        R.IPPE_update_vel_adv(ngrid, fluid, bound)
        gv.incom_iter_count += 1
        if gv.incom_iter_count > config.iter_threshold_max[None]:
            break
    if wc:  # main.py:238-242, enabled
        R.WC_pressure_val(fluid)
        R.WC_pressure_acce(ngrid, fluid, fluid)
        R.WC_pressure_acce(ngrid, fluid, bound)
        R.SPH_advection_update_vel_adv(fluid)
    if fbm:  # main.py:244-250, enabled
        while fluid.general_flag[None] > 0:
            R.SPH_FBM_clean_tmp(fluid)
            R.SPH_FBM_convect(ngrid, fluid, fluid)
            R.SPH_FBM_diffuse(ngrid, fluid, fluid)
            R.SPH_FBM_check_tmp(fluid)
        R.SPH_update_volume_frac(fluid)
    R.SPH_update_mass(fluid)
    R.SPH_update_pos(fluid)
    R.SPH_update_energy(fluid)
    if grid is not None:  # main.py:254, enabled
        R.map_velocity(ngrid, grid, fluid)
    gv.frame_div_iter += gv.div_iter_count
    gv.frame_incom_iter += gv.incom_iter_count


def main(argv):
    if len(argv) >= 3 and argv[0] == "--child":
        _child(argv[1], argv[2])
        return
    scenes = argv or sorted(STEPS)
    for scene in scenes:
        for mode in ("f32", "f64"):
            print("scene %s (%s)" % (scene, mode), flush=True)
            env = dict(os.environ, TAICHI_SHIM_FP=mode)
            subprocess.run([sys.executable, os.path.abspath(__file__), "--child", scene, mode],
                           env=env, check=True)


if __name__ == "__main__":
    main(sys.argv[1:])
