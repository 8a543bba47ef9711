"""Host-side logic that needs no GPU: configuration, emitters, the C ABI library.

* Config constants equal the oracle's reading of the reference's f32 fields.
* The emitters reproduce the initial states the reference's own emitters
  produced (golden ``*.init.npz``) bit for bit.
* The shared library loads and exports every symbol ``include/tichi_sph.h``
  declares (no compute call: this runs without a GPU).
"""
import ctypes
import os
import re

import numpy as np
import pytest

from oracle import sph_oracle as O
from tests import golden_io as G
from tichi_sph_gb300 import sph_config, _native
from tichi_sph_gb300.sph_obj import Fluid

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("scene", G.SCENES)
def test_config_matches_oracle_f32_params(scene):
    cfg = sph_config.load(*G.paths(scene))
    p = O.Params.from_files(*G.paths(scene), taichi_f32=True)
    assert float(cfg.kernel_h[1]) == p.h
    assert float(cfg.kernel_h[2]) == p.h2
    assert float(cfg.kernel_sig[cfg.dim[None]]) == p.sig
    assert cfg.node_num[None] == p.node_num
    np.testing.assert_array_equal(cfg.neighb_grid_coder[None], p.coder)
    np.testing.assert_array_equal(cfg.neighb_search_template, p.template)
    params = cfg.to_params()
    assert params.node_num == p.node_num
    assert params.kernel_h == pytest.approx(p.h, rel=0, abs=0)


@pytest.mark.parametrize("scene", G.SCENES)
def test_emitters_reproduce_reference_initial_state(scene):
    cfg = sph_config.load(*G.paths(scene))
    init, _ = G.load(scene)
    objs = {"fluid": Fluid(cfg.fluid_max_part_num[None], cfg, 0, device="cpu"),
            "bound": Fluid(cfg.bound_max_part_num[None], cfg, 1, device="cpu")}
    for part in cfg.scenario_buffer:
        if part == "sim_env":
            continue
        for prm in cfg.scenario_buffer[part]["objs"]:
            o = objs[part]
            if prm["type"] == "cube":
                o.scene_add_cube(prm["start_pos"], prm["end_pos"], prm["volume_frac"], prm["vel"],
                                 int(prm["color"], 16), prm["particle_relaxing_factor"])
            else:
                o.scene_add_box(prm["start_pos"], prm["end_pos"], prm["layers"], prm["volume_frac"],
                                prm["vel"], int(prm["color"], 16), prm["particle_relaxing_factor"])
    for name, o in objs.items():
        n = int(init[name + "_n"])
        assert o.part_num[None] == n
        for f in ("pos", "vel", "rest_volume"):
            np.testing.assert_array_equal(getattr(o, f)[:n].numpy(), init[name + "_" + f], err_msg=f)
        if scene not in G.FBM_SCENES:  # VFSPH scenes carry harness-added volume-fraction noise
            for f in ("volume_frac", "rest_density", "mass"):
                np.testing.assert_array_equal(getattr(o, f)[:n].numpy(), init[name + "_" + f], err_msg=f)


def test_capacity_overflow_raises():
    cfg = sph_config.load(*G.paths("dfsph2d"))
    f = Fluid(10, cfg, 0, device="cpu")
    with pytest.raises(Exception, match="exceed max_part_num"):
        f.scene_add_cube([0, 0], [0.5, 0.5], [1], [0, 0], 0, 1.0)


def test_bad_config_raises():
    cfg_path, scen_path = G.paths("dfsph2d")
    import json
    cfgd = json.load(open(cfg_path))
    scen = json.load(open(scen_path))
    del cfgd["solver_cs"]
    with pytest.raises(Exception, match="solver_cs"):
        sph_config.Config(cfgd, scen)
    cfgd = json.load(open(cfg_path))
    cfgd["solver_type"] = "WCSPH"
    with pytest.raises(Exception, match="solver_type"):
        sph_config.Config(cfgd, scen)


def test_argv_parsing_accepts_both_spellings():
    assert sph_config.parse_args(["-c", "a.json", "-s", "b.json"]) == ("a.json", "b.json")
    assert sph_config.parse_args(["--configFile=a", "--scenarioFile=b"]) == ("a", "b")


def _declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for fn in os.listdir(inc):
        if fn.endswith(".h"):
            src = open(os.path.join(inc, fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(tsph_[a-z_0-9]+)\s*\(", src))
    return names


def test_library_exports_every_declared_symbol():
    from tichi_sph_gb300 import build
    path = build.build()
    L = ctypes.CDLL(path)
    declared = _declared_symbols()
    assert "tsph_sph_step" in declared and "tsph_create" in declared
    for name in sorted(declared):
        assert hasattr(L, name), name
    # the ctypes signature table covers the same set
    assert declared == set(_native.SIGNATURES), declared ^ set(_native.SIGNATURES)


def test_struct_layouts_match_header():
    # tsph_params / tsph_set / tsph_stats sizes as laid out by the C compiler
    import subprocess
    import tempfile
    src = ('#include <stdio.h>\n#include "tichi_sph.h"\n'
           'int main(){printf("%zu %zu %zu\\n", sizeof(tsph_params), sizeof(tsph_set), sizeof(tsph_stats));return 0;}\n')
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "t")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    assert [int(x) for x in out] == [ctypes.sizeof(_native.Params), ctypes.sizeof(_native.Set),
                                    ctypes.sizeof(_native.Stats)]


def test_map_grid_shape_matches_reference_run():
    """The particle-to-grid Grid (ceil((rt - lb) / dist) per axis) has the shape
    and node positions the golden runs used."""
    from tichi_sph_gb300 import sph_config
    from tichi_sph_gb300.sph_obj import Grid
    from tests import golden_io as G
    for scene in sorted(G.WC_SCENES):
        cfg = sph_config.load(*G.paths(scene))
        _, gold = G.load(scene)
        g = Grid(cfg, device="cpu")
        assert g.shape == tuple(int(x) for x in gold["grid_shape"])
        ref = G.map_grid(gold)
        assert abs(g.dist - ref["dist"]) <= 1e-7 * ref["dist"]
        import numpy as np
        np.testing.assert_allclose(g.pos[(0,) * len(g.shape)].numpy(), ref["lb"], rtol=0, atol=1e-7)


def test_gather_scenes_concatenates_and_rebinds_views():
    """gather_scenes (batched form, host side): every field of every scene lands
    at its scene's offset of the concatenated sets, in scene order, and each
    scene's per-set arrays become views of them (the reference-shaped
    per-scene API reads and writes the batch)."""
    import torch
    from tichi_sph_gb300 import sph_config, workloads
    from tichi_sph_gb300.batch import FIELDS, gather_scenes
    from tichi_sph_gb300.simulation import Simulation
    sims = []
    for c, s in workloads.batched_dambreaks(n_scenes=3, n_min=200, n_max=800):
        sim = Simulation(sph_config.Config(c, s), device="cpu")
        sim.init_scenario()
        sims.append(sim)
    before = [{key: {f: getattr(getattr(s, key), f)[:getattr(s, key).part_num[None]].clone() for f in FIELDS}
               for key in ("fluid", "bound")} for s in sims]
    fluid, bound, nf, nb = gather_scenes(sims, device="cpu")
    assert nf == [s.fluid.part_num[None] for s in sims] and nb == [s.bound.part_num[None] for s in sims]
    assert fluid.part_num[None] == sum(nf) and bound.part_num[None] == sum(nb)
    for big, key, counts in ((fluid, "fluid", nf), (bound, "bound", nb)):
        off = 0
        for i, (s, n) in enumerate(zip(sims, counts)):
            for f in FIELDS:
                assert torch.equal(getattr(big, f)[off:off + n], before[i][key][f]), (key, i, f)
            # a write through the scene's view reaches the batch
            getattr(s, key).pos[0, 0] = 123.0
            assert float(getattr(big, "pos")[off, 0]) == 123.0
            off += n


def test_status_bits_become_warnings_once_per_condition():
    """A step's status bits (TSPH_ST_*) reach the Python user as RuntimeWarnings,
    each condition once per solver; the step itself goes on, as the reference
    does."""
    import warnings
    from tichi_sph_gb300 import _native as N
    both = N.ST_NONFINITE_POS | N.ST_OUTSIDE_GRID
    assert len(N.status_messages(both)) == 2 and N.status_messages(0) == []
    assert len(N.status_messages(N.ST_DIV_ITER_CAP | N.ST_DENS_ITER_CAP | N.ST_FBM_PASS_CAP)) == 3
    w = N.StatusWarner(scene=2)
    with warnings.catch_warnings(record=True) as got:
        warnings.simplefilter("always")
        w(0)
        w(N.ST_OUTSIDE_GRID)
        w(N.ST_OUTSIDE_GRID)            # already reported
        w(both)                         # only the new condition
        w(N.ST_DENS_ITER_CAP)
    msgs = [str(x.message) for x in got]
    assert all(x.category is RuntimeWarning for x in got)
    assert len(msgs) == 3 and all(m.endswith("(scene 2)") for m in msgs)
    assert "outside the neighbour grid" in msgs[0] and "not finite" in msgs[1] and "constant-density" in msgs[2]


class _FakeSet:
    def __init__(self):
        from tichi_sph_gb300.sph_obj import Scalar
        self.compression = Scalar(0.0)
        self.general_flag = Scalar(0)


class _FakeSolver:
    """Records the phase entries a composed step reaches (no GPU)."""

    def __init__(self, fbm=False, compressions=()):
        from tichi_sph_gb300.sph import _Composer
        self.fluid, self.bound = _FakeSet(), _FakeSet()
        self.fbm = fbm
        self.log = []
        self.comp = list(compressions)
        self.flags = [1, 1, 0]
        self.composer = _Composer(self)
        self.fluid._solver = self.bound._solver = self

    def grid_build(self):
        self.log.append("grid")

    def density_alpha(self):
        self.log.append("density")

    def adv_psi(self, kind):
        self.log.append("psi%d" % kind)
        return self.comp.pop(0) if self.comp else 0.0

    def update_vel_adv(self, kind):
        self.log.append("vel%d" % kind)

    def nonpressure(self, terms):
        self.log.append("nonpressure%d" % terms)

    def wc_pressure(self):
        self.log.append("wc")

    def fbm_pass(self):
        self.log.append("fbm")
        return self.flags.pop(0)

    def update(self):
        self.log.append("update")

    def stats(self):
        self.log.append("stats")


def test_composed_step_reaches_the_phase_entries():
    """main.py:175-256 written with the reference-named kernels reaches the
    phase entries in order, one call per group; the Python solver loops follow
    the compression each sweep A reports, and the volume-fraction loop the
    general flag of each pass."""
    from tests.test_gpu_kernel_level import reference_shaped_sph_step
    from tichi_sph_gb300 import Ngrid
    from tichi_sph_gb300.sph_config import load
    from tests import golden_io as G
    cfg = load(*G.paths("vfsph2d"))
    # divergence: 2 iterations (floor); density: a third one while above 1e-3 ... then below
    fake = _FakeSolver(fbm=True, compressions=[0.0, 0.0, 0.5, 0.5, 1e-4])
    ng = Ngrid(cfg)
    ng._solver = fake
    assert reference_shaped_sph_step(cfg, ng, fake.fluid, fake.bound, fbm=True, wc=True) == (2, 3)
    assert fake.log == ["grid", "density", "psi0", "vel0", "psi0", "vel0", "nonpressure7", "psi1", "vel1", "psi1",
                        "vel1", "psi1", "vel1", "wc", "fbm", "fbm", "fbm", "update", "stats"]
    assert fake.fluid.compression[None] == 1e-4 and fake.fluid.general_flag[None] == 0
    fake.log.clear()
    fake.flags = [0]
    reference_shaped_sph_step(cfg, ng, fake.fluid, fake.bound, fbm=True, viscosity=False)
    assert "nonpressure5" in fake.log  # gravity + surface tension, no viscosity


def test_composed_step_incomplete_group_raises():
    from tichi_sph_gb300 import Ngrid, sph as S
    from tichi_sph_gb300._native import TsphError
    fake = _FakeSolver()
    fl, bd = fake.fluid, fake.bound
    ng = Ngrid(None)
    ng._solver = fake
    for f in (ng.clear_node, lambda: ng.encode(fl), lambda: ng.encode(bd), ng.mem_shift, lambda: ng.fill_node(fl),
              lambda: ng.fill_node(bd), lambda: S.SPH_clean_value(fl)):
        f()
    assert fake.log == []  # the grid group waits for its last call
    S.SPH_clean_value(bd)
    assert fake.log == ["grid"] and fl.general_flag[None] == 1
    S.SPH_prepare_attr(ng, fl, fl)
    with pytest.raises(TsphError, match=r"SPH_prepare_attr\(fb\)"):
        S.IPPE_adv_psi_init(fl)
    with pytest.raises(TsphError, match="twice"):
        S.SPH_prepare_attr(ng, fl, fl)
        S.SPH_prepare_attr(ng, fl, fl)
    with pytest.raises(TsphError, match="does not belong"):
        S.SPH_prepare_attr(ng, fl, _FakeSet())
    with pytest.raises(RuntimeError, match="no solver"):
        Ngrid(None).clear_node()
