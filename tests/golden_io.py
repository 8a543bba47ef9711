"""Loading of the committed golden scenes (reference-run fixtures)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SCENES = ["dfsph2d", "dfsph2d_r2", "dfsph3d", "edge2d", "vfsph2d", "vfsph3d", "wcsph2d", "wcsph3d"]
FBM_SCENES = {"vfsph2d", "vfsph3d"}
WC_SCENES = {"wcsph2d", "wcsph3d"}   # weakly compressible block and particle-to-grid map enabled
STATE_IN = ["pos", "vel", "volume_frac", "rest_volume", "mass", "rest_density"]
COMPARED = ["pos", "vel", "vel_adv", "acce", "acce_adv", "mass", "rest_density", "volume_frac",
            "volume_frac_tmp", "W", "sph_density", "sph_compression", "psi_adv", "alpha", "alpha_1",
            "alpha_2", "normal", "drift_vel", "fbm_zeta", "flag", "neighb_cell_seq",
            "neighb_cell_structured_seq"]
WC_COMPARED = ["pressure"]


def paths(scene):
    s = os.path.join(GOLDEN, "scenes", scene)
    return s + ".config.json", s + ".scenario.json"


def load(scene):
    return (np.load(os.path.join(GOLDEN, scene + ".init.npz")),
            np.load(os.path.join(GOLDEN, scene + ".steps.npz")))


def init_arrays(init, which):
    return {k: init[which + "_" + k] for k in STATE_IN}


def n_steps(steps):
    n = 0
    while "s%d_dt" % n in steps:
        n += 1
    return n


def map_grid(steps):
    """The particle-to-grid map's Grid of a WC scene: dict(lb, dist, shape)."""
    return {"lb": steps["grid_lb"], "dist": float(steps["grid_dist"]), "shape": tuple(int(x) for x in steps["grid_shape"])}
