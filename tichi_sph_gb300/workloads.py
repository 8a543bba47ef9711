"""Benchmark scenes written in the reference's config / scenario JSON schema.

Seeded synthetic stand-ins for the benchmark configurations (the reference
publishes none): lattice blocks and boxes emitted by the reference's own emitter
rules (``sph_obj.py:102-163``).

* :func:`dambreak_2d` -- 2D single-phase DFSPH dam break: fluid 1.0 x 2.0 m at
  0.02 m (50 x 100 = 5,000 particles) in a 4 x 4 m box with 3 boundary layers,
  rest density 1000, gravity -9.81, viscosity 0.01, dt 1e-3 (``solver_cs`` 20:
  dt = part_size / cs, CFL always on), tolerances 0.1% / 1%.
* :func:`dambreak_3d` -- 3D single-phase DFSPH dam break: a 1 m cube at 0.01 m
  (100^3 = 1,000,000 particles) in the x-min corner of a 3 x 1.5 x 1 m tank
  (x, y up, z) with 3 boundary layers (566,742 particles), h = 0.02, rest density
  1000, viscosity 0.01, ``solver_cs`` 50 so dt <= 2e-4 with CFL factor 0.5,
  tolerances 0.1% / 1%.
"""


def _config(solver="DFSPH", cs=50, div_tol=1e-2, comp_tol=1e-3, gamma=0.0, fbm_c=0.0, fbm_d=0.0):
    return {
        "arch": "gpu", "device_memory_GB": 6,
        "solver_type": solver, "solver_wc_gamma": 7,
        "solver_divergence_threshold": div_tol, "solver_compression_threshold": comp_tol,
        "solver_iter_threshold_min": 2, "solver_iter_threshold_max": 100,
        "solver_if_cfl": True, "solver_cs": cs, "solver_cfl_factor": 0.5,
        "solver_neighb_range": 1, "solver_neighb_grid_size_TO_global_part_size": 2,
        "solver_fbm_diffusion_term": fbm_d, "solver_fbm_convection_term": fbm_c,
        "solver_surface_tension_gamma": gamma,
        "gui_res": [1080, 1080], "gui_part_zoomer": 1.0, "gui_fps": 30,
        "gui_canvas_bgcolor": [0.2, 0.2, 0.6], "gui_camera_pos": [6.0, 1.0, 0.0],
        "gui_camera_lookat": [0.0, 0.0, 0.0],
    }


def _obj(kind, start, end, vf, vel, rf=1.0, layers=None):
    o = {"type": kind, "vel": vel, "particle_relaxing_factor": rf, "start_pos": start, "end_pos": end,
         "volume_frac": vf, "color": "0x6F7DBC"}
    if layers is not None:
        o["layers"] = layers
    return o


def dambreak_2d():
    cfg = _config(cs=20)
    scen = {
        "sim_env": {"global_part_size": 0.02, "global_dynamic_viscosity": 0.01, "sim_dim": 2,
                    "sim_space_lb": [-0.2, -0.2], "sim_space_rt": [4.2, 4.2], "gravity": [0, -9.81],
                    "phase_num": 1, "phase_rest_density": [1000], "phase_color_hex": ["0x6F7DBC"]},
        "fluid": {"max_part_num": 5000, "objs": [_obj("cube", [0.0, 0.0], [1.0, 2.0], [1], [0, 0])]},
        "bound": {"max_part_num": 4000, "objs": [_obj("box", [-0.07, -0.07], [3.93, 3.93], [1], [0, 0], layers=3)]},
    }
    return cfg, scen


def dambreak_3d(n_side=100, spacing=0.01):
    """A cube of n_side^3 fluid particles; n_side = 100 is the 1M-particle case."""
    L = n_side * spacing
    cfg = _config(cs=50)
    scen = {
        "sim_env": {"global_part_size": spacing, "global_dynamic_viscosity": 0.01, "sim_dim": 3,
                    "sim_space_lb": [-0.15, -0.15, -0.15], "sim_space_rt": [3.2, 2.0, 1.2],
                    "gravity": [0, -9.81, 0], "phase_num": 1, "phase_rest_density": [1000],
                    "phase_color_hex": ["0x6F7DBC"]},
        "fluid": {"max_part_num": n_side ** 3, "objs": [_obj("cube", [0.0, 0.0, 0.0], [L, L, L], [1], [0, 0, 0])]},
        "bound": {"max_part_num": _tank_bound_cap(spacing), "objs": [
            _obj("box", [-0.035, -0.035, -0.035], [3.035, 1.535, 1.035], [1], [0, 0, 0], layers=3)]},
    }
    return cfg, scen


def _tank_bound_cap(spacing):
    """Boundary capacity of the 3 x 1.5 x 1 m tank: 566,742 particles at 0.01 m,
    scaled with the wall area per particle (plus 5%) at other spacings."""
    return 566742 if spacing == 0.01 else int(566742 * (0.01 / spacing) ** 2 * 1.05)


def twophase_3d(n_side=100, spacing=0.01, seed=3):
    """3D two-phase VFSPH: two 1 m cubes side by side (rest densities 1000 and 500)
    in the 3 x 1.5 x 1 m tank, surface tension 0.07, the volume-fraction update on.
    The reference has one global viscosity (sph.py:129): 0.01 stands for the
    0.01 / 0.05 pair.  Returns (config, scenario, volume-fraction noise function)."""
    import numpy as np
    L = n_side * spacing
    cfg = _config(solver="VFSPH", cs=50, gamma=0.07, fbm_c=50.0, fbm_d=0.0)
    scen = {
        "sim_env": {"global_part_size": spacing, "global_dynamic_viscosity": 0.01, "sim_dim": 3,
                    "sim_space_lb": [-0.15, -0.15, -0.15], "sim_space_rt": [3.2, 2.0, 1.2],
                    "gravity": [0, -9.81, 0], "phase_num": 2, "phase_rest_density": [1000, 500],
                    "phase_color_hex": ["0x6F7DBC", "0xFA8012"]},
        "fluid": {"max_part_num": 2 * n_side ** 3, "objs": [
            _obj("cube", [0.0, 0.0, 0.0], [L, L, L], [1, 0], [0, 0, 0]),
            _obj("cube", [L + spacing, 0.0, 0.0], [2 * L + spacing, L, L], [0, 1], [0, 0, 0])]},
        "bound": {"max_part_num": 566742, "objs": [
            _obj("box", [-0.035, -0.035, -0.035], [3.035, 1.535, 1.035], [1, 0], [0, 0, 0], layers=3)]},
    }

    def noise(vf):
        """Seeded U(-0.05, 0.05) on phase 0, clipped to [0, 1]; phase 1 = 1 - phase 0."""
        rng = np.random.default_rng(seed)
        v0 = np.clip(vf[:, 0] + rng.uniform(-0.05, 0.05, len(vf)), 0.0, 1.0).astype(np.float32)
        out = np.stack([v0, (1.0 - v0).astype(np.float32)], axis=1)
        return out
    return cfg, scen, noise


def batched_dambreaks(n_scenes=256, seed=4, spacing=0.01, n_min=2000, n_max=200000):
    """Independent 3D dam breaks of uneven size: fluid counts log-uniform in
    [n_min, n_max], block aspect ratios x/y and z/y uniform in [0.5, 2], rest
    density uniform in [800, 1200], each block in the x-min corner of its own tank
    (2.5 x 1.5 x 1 block lengths, 3 boundary layers).  Returns a list of
    (config, scenario) pairs."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_scenes):
        n = float(np.exp(rng.uniform(np.log(n_min), np.log(n_max))))
        ax, az = rng.uniform(0.5, 2.0), rng.uniform(0.5, 2.0)
        ny = max(2, int(round((n / (ax * az)) ** (1.0 / 3.0))))
        nx, nz = max(2, int(round(ax * ny))), max(2, int(round(az * ny)))
        Lx, Ly, Lz = nx * spacing, ny * spacing, nz * spacing
        rho = float(rng.uniform(800.0, 1200.0))
        t = 3.5 * spacing
        box_lo = [-t, -t, -t]
        box_hi = [2.5 * Lx + t, 1.5 * Ly + t, Lz + t]
        # boundary count with the emitter's arithmetic (sph_obj.py:102-107, 140-151)
        sp32 = float(np.float32(spacing))
        shape = ((np.array(box_hi, np.float32) - np.array(box_lo, np.float32) + 1e-7) / sp32).astype(np.int32)
        n_box = int(np.prod(shape.astype(np.int64)) - np.prod(np.maximum(shape.astype(np.int64) - 6, 0)))
        cfg = _config(cs=50)
        scen = {
            "sim_env": {"global_part_size": spacing, "global_dynamic_viscosity": 0.01, "sim_dim": 3,
                        "sim_space_lb": [b - 0.1 for b in box_lo],
                        "sim_space_rt": [box_hi[0] + 0.1, box_hi[1] + 0.1 + 0.5 * Ly, box_hi[2] + 0.1],
                        "gravity": [0, -9.81, 0], "phase_num": 1, "phase_rest_density": [rho],
                        "phase_color_hex": ["0x6F7DBC"]},
            "fluid": {"max_part_num": nx * ny * nz, "objs": [
                _obj("cube", [0.0, 0.0, 0.0], [Lx, Ly, Lz], [1], [0, 0, 0])]},
            "bound": {"max_part_num": n_box, "objs": [
                _obj("box", box_lo, box_hi, [1], [0, 0, 0], layers=3)]},
        }
        out.append((cfg, scen))
    return out


def diff_block(nx=46, ny=46, nz=47, spacing=0.01, seed=5, v_std=0.1, fixed_iters=None, relax=1.0, gamma=0.0):
    """Differentiable DFSPH scene: a block of nx*ny*nz fluid particles (46 x 46 x 47
    = 99,452 by default) in the x/z-min corner of a tank 1.6 x 1.5 x 1.6 block
    lengths with 3 boundary layers, dt = 5e-4 (``solver_cs`` 20; the CFL limit
    binds only above 10 m/s), tolerances 1% / 0.1%.  ``fixed_iters`` = k makes
    both solves run exactly k iterations (tolerances out of reach).  Returns
    (config, scenario, initial-velocity function, target point); ``relax`` < 1
    emits the same lattice at relax x spacing (a compressed block).  Velocities are
    seeded N(0, v_std) per component, the target is the block's centre plus a
    seeded U(-0.05, 0.05) offset per axis; ``gamma`` is the surface-tension
    coefficient."""
    import numpy as np
    Lx, Ly, Lz = nx * spacing, ny * spacing, nz * spacing
    t = 3.5 * spacing
    box_lo = [-t, -t, -t]
    box_hi = [1.6 * Lx + t, 1.5 * Ly + t, 1.6 * Lz + t]
    sp32 = float(np.float32(spacing))
    shape = ((np.array(box_hi, np.float32) - np.array(box_lo, np.float32) + 1e-7) / sp32).astype(np.int32)
    n_box = int(np.prod(shape.astype(np.int64)) - np.prod(np.maximum(shape.astype(np.int64) - 6, 0)))
    if fixed_iters:
        cfg = _config(cs=20, div_tol=1e9, comp_tol=1e9, gamma=gamma)
        cfg["solver_iter_threshold_min"] = int(fixed_iters)
    else:
        cfg = _config(cs=20, gamma=gamma)
    scen = {
        "sim_env": {"global_part_size": spacing, "global_dynamic_viscosity": 0.01, "sim_dim": 3,
                    "sim_space_lb": [b - 0.1 for b in box_lo],
                    "sim_space_rt": [box_hi[0] + 0.1, box_hi[1] + 0.1, box_hi[2] + 0.1],
                    "gravity": [0, -9.81, 0], "phase_num": 1, "phase_rest_density": [1000],
                    "phase_color_hex": ["0x6F7DBC"]},
        "fluid": {"max_part_num": nx * ny * nz, "objs": [
            _obj("cube", [0.0, 0.0, 0.0], [Lx * relax, Ly * relax, Lz * relax], [1], [0, 0, 0], rf=relax)]},
        "bound": {"max_part_num": n_box, "objs": [_obj("box", box_lo, box_hi, [1], [0, 0, 0], layers=3)]},
    }
    rng = np.random.default_rng(seed)
    target = np.array([0.5 * Lx, 0.5 * Ly, 0.5 * Lz]) + rng.uniform(-0.05, 0.05, 3)

    def velocities(n):
        r = np.random.default_rng(seed + 1)
        return (r.standard_normal((n, 3)) * v_std).astype(np.float32)
    return cfg, scen, velocities, target
