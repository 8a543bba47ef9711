"""The reference-structured C restatement (the timed CPU baseline) against the
FP64 oracle on the golden scenes: FP32 vs FP64, one substep from the reference
state, identical iteration counts, fields within 1e-4 of their scale."""
import numpy as np
import pytest

from oracle import sph_oracle as O
from oracle.port import PortSim
from tests import golden_io as G
from tichi_sph_gb300 import sph_config


@pytest.mark.parametrize("scene", G.SCENES)
def test_port_one_step(scene):
    init, gold = G.load(scene)
    cfg = sph_config.load(*G.paths(scene))
    fa, ba = G.init_arrays(init, "fluid"), G.init_arrays(init, "bound")
    sim = PortSim(cfg, fa, ba, fbm=scene in G.FBM_SCENES)
    st = sim.substep()
    p = O.Params.from_files(*G.paths(scene), taichi_f32=True)
    fl, bd = O.sets_from_arrays(p, {k: v.astype(np.float64) for k, v in fa.items()},
                                {k: v.astype(np.float64) for k, v in ba.items()})
    ost = O.run_substep(fl, bd, p, O.Stats(), fbm=scene in G.FBM_SCENES)
    assert (st["div_iter"], st["incom_iter"]) == (ost.div_iter, ost.incom_iter)
    dens = float(np.abs(fl.sph_density).max())
    for f in ("pos", "vel", "sph_density", "psi_adv", "alpha", "volume_frac"):
        a = getattr(sim.fluid, f).astype(np.float64)
        b = np.asarray(getattr(fl, f)).reshape(a.shape)
        scale = max(float(np.abs(b).max()), dens if f == "psi_adv" else 0.0)
        assert np.abs(a - b).max() <= 1e-4 * scale, (scene, f)
    sim.close()
