"""Coincident fluid particles under surface tension (needs a GPU).

The reference's surface-tension pass (sph.py:152-166) leaves out pairs at
r = 0.  The CUDA curvature loop visits every candidate of the template cells
without a position test and relies on the terms it should leave out being
exactly zero: a particle's own (n_i - n_i) and that of a particle at its exact
position, whose normal is the same bit for bit (the two have the same
neighbours in the same order, each leaving the other out).  Here a phase-0
particle of the two-phase golden scene (gamma 0.07) gets a twin at its exact
position: one substep meets the one-step bar against the FP64 oracle, whose
loops test r > 0, and the twins' normals and accelerations are bitwise equal.
"""
import numpy as np
import pytest

from oracle import sph_oracle as O
from tests import golden_io as G
from tests.test_gpu_parity import _fluid_fields, _need_cuda, compare, make_gpu, make_oracle

pytestmark = pytest.mark.gpu

SCENE = "vfsph3d"


@pytest.mark.parametrize("tpp", [1, 4])
def test_coincident_twin_under_surface_tension(tpp):
    _need_cuda()
    init, _ = G.load(SCENE)
    fa, ba = G.init_arrays(init, "fluid"), G.init_arrays(init, "bound")
    vf0 = np.asarray(fa["volume_frac"])[:, 0]
    pos = np.asarray(fa["pos"], dtype=np.float64)
    # the phase-0 particle nearest the phase-0 block's centre (surface tension on)
    cand = np.where(vf0 > 0.99)[0]
    k = int(cand[np.argmin(np.linalg.norm(pos[cand] - pos[cand].mean(axis=0), axis=1))])
    twin = {key: np.concatenate([np.asarray(v), np.asarray(v)[k:k + 1]]) for key, v in fa.items()}
    n = len(twin["pos"])
    cfg, fl, bd, solver = make_gpu(SCENE, twin, ba)
    solver.set_threads_per_particle(tpp)
    p, ofl, obd = make_oracle(SCENE, twin, ba)
    try:
        solver.substep()
        gs = solver.stats()
        st = O.run_substep(ofl, obd, p, O.Stats(), fbm=SCENE in G.FBM_SCENES)
        assert (gs["div_iter"], gs["incom_iter"]) == (st.div_iter, st.incom_iter)
        dens = float(np.abs(ofl.sph_density).max(initial=0.0))
        fdt = st.dt if SCENE in G.FBM_SCENES else None
        compare(SCENE, "twin tpp%d" % tpp, fl, ofl, _fluid_fields(SCENE, p), dens_scale=dens, fbm_dt=fdt)
        for f in ("normal", "acce_adv", "vel", "pos"):
            a = getattr(fl, f)[:n].cpu().numpy()
            np.testing.assert_array_equal(a[k], a[n - 1], err_msg=f)
        assert np.abs(getattr(fl, "normal")[k].cpu().numpy()).max() > 0
    finally:
        solver.close()
