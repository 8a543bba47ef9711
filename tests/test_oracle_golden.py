"""The FP64 oracle against golden vectors recorded from the reference's own kernels.

The golden runs store f64 fields, so the oracle (a restatement of the same
algorithm in f64) must agree to summation-order rounding: 1e-11 of each field's
scale (the scale of psi_adv is the density it was cancelled from), and the
solver iteration counts, FBM flags and cell codes must be identical.
"""
import numpy as np
import pytest

from oracle import sph_oracle as O
from tests import golden_io as G

RTOL = 1e-11


@pytest.mark.parametrize("scene", G.SCENES)
def test_oracle_matches_reference_run(scene):
    p = O.Params.from_files(*G.paths(scene))
    init, gold = G.load(scene)
    fl, bd = O.sets_from_arrays(p, G.init_arrays(init, "fluid"), G.init_arrays(init, "bound"))
    st = O.Stats()
    wc = scene in G.WC_SCENES
    for s in range(G.n_steps(gold)):
        mg = G.map_grid(gold) if wc else None
        O.run_substep(fl, bd, p, st, fbm=scene in G.FBM_SCENES, wc=wc, map_grid=mg)
        pre = "s%d_" % s
        if wc:
            g = gold[pre + "grid_vel"]
            assert float(np.abs(mg["vel"] - g).max()) <= RTOL * max(float(np.abs(g).max()), 1e-12), (scene, s)
        assert st.div_iter == int(gold[pre + "div_iter"])
        assert st.incom_iter == int(gold[pre + "incom_iter"])
        assert st.dt == pytest.approx(float(gold[pre + "dt"]), rel=1e-14)
        assert st.time_count == pytest.approx(float(gold[pre + "time_count"]), rel=1e-14)
        for key, val in (("compression", fl.compression),
                         ("kinetic_energy", fl.statistics_kinetic_energy),
                         ("potential_energy", fl.statistics_gravity_potential_energy)):
            g = float(gold[pre + key])
            # compression is a mean of psi_adv / rest_psi: its scale is O(1)
            floor = 1.0 if key == "compression" else 1e-12
            assert abs(val - g) <= RTOL * max(abs(g), floor), key
        for name, obj in (("fluid", fl), ("bound", bd)):
            dens_scale = float(np.abs(gold[pre + name + "_sph_density"]).max(initial=0.0))
            for f in G.COMPARED + (G.WC_COMPARED if wc and name == "fluid" else []):
                a = np.asarray(getattr(obj, f), dtype=np.float64)
                b = gold[pre + name + "_" + f].astype(np.float64)
                if f in ("flag", "neighb_cell_seq", "neighb_cell_structured_seq"):
                    np.testing.assert_array_equal(a, b, err_msg="%s %s %s" % (scene, name, f))
                    continue
                scale = float(np.abs(b).max(initial=0.0))
                if f == "psi_adv":
                    scale = max(scale, dens_scale)
                err = float(np.abs(a - b).max(initial=0.0))
                assert err <= RTOL * max(scale, 1e-12), (scene, s, name, f, err, scale)


def test_kernel_known_answers():
    """Analytic checks of W / W_grad (sph_util.py:16-37) independent of any run."""
    p = O.Params.from_files(*G.paths("dfsph3d"))
    assert O.W(np.array([0.0]), p)[0] == pytest.approx(8 / np.pi / p.h ** 3)
    # continuity at q = 0.5 and compact support at q >= 1
    h = p.h
    assert O.W(np.array([0.5 * h - 1e-12]), p)[0] == pytest.approx(O.W(np.array([0.5 * h + 1e-12]), p)[0], rel=1e-9)
    assert O.W_grad(np.array([0.5 * h - 1e-12]), p)[0] == pytest.approx(
        O.W_grad(np.array([0.5 * h + 1e-12]), p)[0], rel=1e-9)
    assert O.W(np.array([h, 1.5 * h]), p).tolist() == [0.0, 0.0]
    assert O.W_grad(np.array([h]), p)[0] == 0.0
    # integral of W over its support is 1 (3D lattice quadrature)
    dx = h / 40
    ax = np.arange(-h, h + dx / 2, dx)
    X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
    r = np.sqrt(X ** 2 + Y ** 2 + Z ** 2).ravel()
    assert np.sum(O.W(r, p)) * dx ** 3 == pytest.approx(1.0, rel=2e-3)
    p2 = O.Params.from_files(*G.paths("dfsph2d"))
    assert O.W(np.array([0.0]), p2)[0] == pytest.approx(40 / 7 / np.pi / p2.h ** 2)
    ax = np.arange(-p2.h, p2.h + p2.h / 400, p2.h / 200)
    X, Y = np.meshgrid(ax, ax, indexing="ij")
    r = np.sqrt(X ** 2 + Y ** 2).ravel()
    assert np.sum(O.W(r, p2)) * (p2.h / 200) ** 2 == pytest.approx(1.0, rel=2e-3)
