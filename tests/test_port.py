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


@pytest.mark.parametrize("scene", G.SCENES)
def test_port_fp64_one_step(scene):
    """The FP64 build of the restatement (the one-step oracle at the benchmark
    sizes) against the numpy oracle: both compute and store every field in FP64
    within a substep, so they differ by the FP32 rounding of the returned arrays
    and by summation order: identical iteration counts, every compared field
    within 2e-7 of its scale."""
    init, gold = G.load(scene)
    cfg = sph_config.load(*G.paths(scene))
    fa, ba = G.init_arrays(init, "fluid"), G.init_arrays(init, "bound")
    sim = PortSim(cfg, fa, ba, fbm=scene in G.FBM_SCENES, fp64=True)
    st = sim.substep()
    p = O.Params.from_files(*G.paths(scene), taichi_f32=True)
    fl, bd = O.sets_from_arrays(p, {k: v.astype(np.float64) for k, v in fa.items()},
                                {k: v.astype(np.float64) for k, v in ba.items()})
    ost = O.run_substep(fl, bd, p, O.Stats(), fbm=scene in G.FBM_SCENES)
    assert (st["div_iter"], st["incom_iter"]) == (ost.div_iter, ost.incom_iter)
    assert st["dt"] == pytest.approx(ost.dt, rel=1e-12)
    assert st["compression"] == pytest.approx(fl.compression, rel=1e-5, abs=1e-9)
    dens = float(np.abs(fl.sph_density).max())
    for f in ("pos", "vel", "vel_adv", "sph_density", "W", "psi_adv", "alpha", "alpha_1", "alpha_2",
              "volume_frac", "normal"):
        a = getattr(sim.fluid, f).astype(np.float64)
        b = np.asarray(getattr(fl, f)).reshape(a.shape)
        scale = max(float(np.abs(b).max()), dens if f == "psi_adv" else 0.0)
        assert np.abs(a - b).max() <= 2e-7 * max(scale, 1e-30), (scene, f, np.abs(a - b).max(), scale)
    sim.close()


@pytest.mark.parametrize("scene", ["dfsph3d", "vfsph3d"])
def test_port_runs_are_bitwise_repeatable(scene):
    """The C restatement fills each cell in id order and sums the compression
    serially, so two runs give the same bits on any thread count (the long runs
    compare the CUDA path against it over 1,000 substeps); its in-cell slots are
    the id-ordered ranks of the reference's combined grid (fluid first)."""
    init, _ = G.load(scene)
    cfg = sph_config.load(*G.paths(scene))
    fa, ba = G.init_arrays(init, "fluid"), G.init_arrays(init, "bound")
    runs = []
    for _ in range(2):
        sim = PortSim(cfg, fa, ba, fbm=scene in G.FBM_SCENES)
        stats = [sim.substep() for _ in range(8)]
        runs.append((stats, {k: v.copy() for k, v in sim.fluid.a.items()}, {k: v.copy() for k, v in sim.bound.a.items()}))
        sim.close()
    (s0, f0, b0), (s1, f1, b1) = runs
    assert s0 == s1
    for a, b in ((f0, f1), (b0, b1)):
        for k in a:
            np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    # in-cell slots: a cell's fluid particles in id order, then its boundary particles in id order
    codes = np.concatenate([f0["neighb_cell_seq"], b0["neighb_cell_seq"]])
    slots = np.concatenate([f0["neighb_in_cell_seq"], b0["neighb_in_cell_seq"]])
    for code in np.unique(codes[codes > 0]):
        idx = np.where(codes == code)[0]          # fluid ids first, each set in id order
        s = slots[idx]
        assert np.all(np.diff(s) == 1), (scene, code)
