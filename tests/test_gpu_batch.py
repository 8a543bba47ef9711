"""Batched form against the same scenes stepped one at a time (needs a GPU).

A scene in a batch keeps its own constants, time step, solver loops and
summation order, so after every substep its state must equal -- bit for bit --
the state of the same scene stepped alone through the plain path.  The batches
mix scene sizes, rest densities, boxes, velocities and an empty fluid set.
"""
import types

import numpy as np
import pytest
import torch

from tests import golden_io as G

pytestmark = pytest.mark.gpu


def _need_cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _variant(scene, k):
    """Scene k of a batch built from golden scene `scene`: (config, fluid arrays, bound arrays)."""
    from tichi_sph_gb300 import sph_config
    import json
    cpath, spath = G.paths(scene)
    cfgd, scen = json.load(open(cpath)), json.load(open(spath))
    init, _ = G.load(scene)
    fa = {key: np.array(v) for key, v in G.init_arrays(init, "fluid").items()}
    ba = {key: np.array(v) for key, v in G.init_arrays(init, "bound").items()}
    if k == 1:  # fewer particles, faster and reversed flow, denser phase
        keep = np.arange(len(fa["pos"])) % 3 != 0
        fa = {key: v[keep] for key, v in fa.items()}
        fa["vel"] = -1.5 * fa["vel"]
        scen["sim_env"]["phase_rest_density"] = [x * 1.1 for x in scen["sim_env"]["phase_rest_density"]]
    elif k == 2:  # the whole scene translated, with its sim space
        shift = np.array([0.37, -0.21, 0.13][: len(fa["pos"][0])], dtype=np.float32)
        fa["pos"] = fa["pos"] + shift
        ba["pos"] = ba["pos"] + shift
        for key in ("sim_space_lb", "sim_space_rt"):
            scen["sim_env"][key] = [float(np.float32(a) + s) for a, s in zip(scen["sim_env"][key], shift)]
    elif k == 3:  # no fluid at all
        fa = {key: v[:0] for key, v in fa.items()}
    cfgd["solver_cs"] = cfgd["solver_cs"] + 10 * k
    return sph_config.Config(cfgd, scen), fa, ba


def _solo(cfg, fa, ba, fbm):
    from tichi_sph_gb300 import Fluid, Solver
    objs = []
    for uid, arrs in enumerate((fa, ba)):
        n = len(arrs["pos"])
        o = Fluid(max(n, 1), cfg, uid, device="cuda")
        o.part_num[None] = n
        for key, v in arrs.items():
            getattr(o, key)[:n] = torch.as_tensor(np.asarray(v, np.float32), device="cuda").reshape(getattr(o, key)[:n].shape)
        objs.append(o)
    return objs[0], objs[1], Solver(cfg, objs[0], objs[1], fbm=fbm)


@pytest.mark.parametrize("scene,ks", [("dfsph3d", [0, 1, 2, 3]), ("vfsph2d", [0, 1, 2]), ("edge2d", [1, 0])])
def test_batch_equals_scenes_alone(scene, ks):
    _need_cuda()
    from tichi_sph_gb300.batch import BatchSolver, gather_scenes
    fbm = scene in G.FBM_SCENES
    variants = [_variant(scene, k) for k in ks]
    # plain path, one scene at a time
    solo = []
    for cfg, fa, ba in variants:
        fl, bd, s = _solo(cfg, fa, ba, fbm)
        rec = []
        for _ in range(3):
            s.substep()
            st = s.stats()
            rec.append((fl.pos[:len(fa["pos"])].cpu().numpy().copy(), fl.vel[:len(fa["pos"])].cpu().numpy().copy(),
                        fl.sph_density[:len(fa["pos"])].cpu().numpy().copy(),
                        fl.volume_frac[:len(fa["pos"])].cpu().numpy().copy(),
                        bd.sph_density[:len(ba["pos"])].cpu().numpy().copy(), st))
        s.close()
        solo.append(rec)
    # the same scenes in one batch
    sims = []
    for cfg, fa, ba in variants:
        fl, bd, s = _solo(cfg, fa, ba, fbm)
        s.close()
        sims.append(types.SimpleNamespace(config=cfg, fluid=fl, bound=bd))
    fluid, bound, nf, nb = gather_scenes(sims)
    batch = BatchSolver([v[0] for v in variants], fluid, bound, nf, nb, fbm=fbm)
    for step in range(3):
        batch.substep()
        stats = batch.stats()
        for i, sim in enumerate(sims):
            pos, vel, rho, vf, brho, st = solo[i][step]
            n, m = nf[i], nb[i]
            np.testing.assert_array_equal(sim.fluid.pos[:n].cpu().numpy(), pos, err_msg="scene %d pos" % i)
            np.testing.assert_array_equal(sim.fluid.vel[:n].cpu().numpy(), vel, err_msg="scene %d vel" % i)
            np.testing.assert_array_equal(sim.fluid.sph_density[:n].cpu().numpy(), rho)
            np.testing.assert_array_equal(sim.fluid.volume_frac[:n].cpu().numpy(), vf)
            np.testing.assert_array_equal(sim.bound.sph_density[:m].cpu().numpy(), brho)
            for key in ("dt", "time_count", "div_iter", "incom_iter", "fbm_passes", "kinetic_energy",
                        "potential_energy"):
                a, b = stats[i][key], st[key]
                assert (a == b) or (np.isnan(a) and np.isnan(b)), (i, step, key, a, b)
            c1, c2 = stats[i]["compression"], st["compression"]
            assert (c1 == c2) or (np.isnan(c1) and np.isnan(c2)), (i, step, c1, c2)
    batch.close()


def test_batch_moved_boundary_in_one_scene():
    """The boundary sums kept across substeps are per scene: after the caller
    moves a boundary particle of one scene (and changes another's mass), that
    scene's sums are recomputed and the others' kept, and every scene still
    equals its solo run bit for bit."""
    _need_cuda()
    from tichi_sph_gb300.batch import BatchSolver, gather_scenes
    variants = [_variant("dfsph3d", k) for k in (0, 1, 2)]
    moved = 1

    def touch(cfg, bd):
        bd.pos[0, 0] += 0.25 * float(cfg.part_size[1])
        bd.mass[1] *= 1.5

    solo = []
    for i, (cfg, fa, ba) in enumerate(variants):
        fl, bd, s = _solo(cfg, fa, ba, False)
        rec = []
        for step in range(4):
            if step == 2 and i == moved:
                touch(cfg, bd)
            s.substep()
            st = s.stats()
            rec.append((fl.pos[:len(fa["pos"])].cpu().numpy().copy(), fl.vel[:len(fa["pos"])].cpu().numpy().copy(),
                        bd.sph_density[:len(ba["pos"])].cpu().numpy().copy(),
                        bd.sph_compression[:len(ba["pos"])].cpu().numpy().copy(), st))
        s.close()
        solo.append(rec)
    sims = []
    for cfg, fa, ba in variants:
        fl, bd, s = _solo(cfg, fa, ba, False)
        s.close()
        sims.append(types.SimpleNamespace(config=cfg, fluid=fl, bound=bd))
    fluid, bound, nf, nb = gather_scenes(sims)
    batch = BatchSolver([v[0] for v in variants], fluid, bound, nf, nb)
    for step in range(4):
        if step == 2:
            touch(variants[moved][0], sims[moved].bound)
        batch.substep()
        stats = batch.stats()
        for i, sim in enumerate(sims):
            pos, vel, brho, bcomp, st = solo[i][step]
            n, m = nf[i], nb[i]
            tag = "scene %d step %d" % (i, step)
            np.testing.assert_array_equal(sim.fluid.pos[:n].cpu().numpy(), pos, err_msg=tag + " pos")
            np.testing.assert_array_equal(sim.fluid.vel[:n].cpu().numpy(), vel, err_msg=tag + " vel")
            np.testing.assert_array_equal(sim.bound.sph_density[:m].cpu().numpy(), brho, err_msg=tag + " bound rho")
            np.testing.assert_array_equal(sim.bound.sph_compression[:m].cpu().numpy(), bcomp,
                                          err_msg=tag + " bound compression")
            for key in ("dt", "div_iter", "incom_iter", "compression", "kinetic_energy"):
                assert stats[i][key] == st[key], (tag, key, stats[i][key], st[key])
    batch.close()
