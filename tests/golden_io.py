"""Loading of the committed golden scenes (reference-run fixtures)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SCENES = ["dfsph2d", "dfsph2d_r2", "dfsph3d", "edge2d", "vfsph2d", "vfsph3d"]
FBM_SCENES = {"vfsph2d", "vfsph3d"}
STATE_IN = ["pos", "vel", "volume_frac", "rest_volume", "mass", "rest_density"]
COMPARED = ["pos", "vel", "vel_adv", "acce", "acce_adv", "mass", "rest_density", "volume_frac",
            "volume_frac_tmp", "W", "sph_density", "sph_compression", "psi_adv", "alpha", "alpha_1",
            "alpha_2", "normal", "drift_vel", "fbm_zeta", "flag", "neighb_cell_seq",
            "neighb_cell_structured_seq"]


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
