"""CUDA path against the FP64 oracle, through the C ABI (needs a GB300).

Inputs are the golden scenes' initial states (emitted by the reference's own
code) and, for the one-step cases, the reference-run golden state after each
step, rounded to f32.  The oracle is configured with the same f32 constants the
CUDA path uses (``Params(..., taichi_f32=True)``).

Tolerances (written per field below): the CUDA path computes in FP32 like the
reference, the oracle in FP64.  Each field's error is max|cuda - oracle| divided
by the field's scale max|oracle|; ``psi_adv`` is a difference of densities, so
its scale is the density it was cancelled from.  One step from identical inputs:
1e-5 for density, psi_adv, alpha, velocities, positions, volume fractions (the
bar of the hot-path spec; a position's error is its velocity's error times dt),
2e-6 for masses; cell codes, flags and solver iteration counts exactly equal.  With the volume-fraction update on,
``acce_adv`` is overwritten by (v_adv - vel) / dt (sph.py:332), a difference of
two velocities, so it and the quantities built from it (``acce``, ``drift_vel``)
are scaled by the velocity they were differenced from (max|v_adv| / dt, and
max|v_adv| for ``drift_vel`` which carries a factor dt); ``volume_frac_tmp`` is an
increment of ``volume_frac`` and is scaled by it.  With the weakly compressible
block on (``wcsph*`` scenes) the fluid's ``pressure`` is compared too, and the
particle-to-grid map's node velocities (1e-5 of their largest magnitude).
"""
import numpy as np
import pytest
import torch

from oracle import sph_oracle as O
from tests import golden_io as G

pytestmark = pytest.mark.gpu

TOL_ONE_STEP = {
    "pos": 1e-5, "vel": 1e-5, "vel_adv": 1e-5, "acce_adv": 1e-5, "mass": 2e-6, "rest_density": 2e-6,
    "volume_frac": 1e-5, "volume_frac_tmp": 1e-5, "W": 1e-5, "sph_density": 1e-5,
    "sph_compression": 1e-5, "psi_adv": 1e-5, "alpha": 1e-5, "alpha_1": 1e-5, "alpha_2": 1e-5,
    "normal": 1e-5, "drift_vel": 1e-5, "fbm_zeta": 1e-5, "acce": 1e-5, "pressure": 1e-5,
}
EXACT = ("neighb_cell_seq", "neighb_cell_structured_seq", "flag")
BOUND_FIELDS = ("W", "sph_density", "sph_compression", "alpha_2", "alpha", "neighb_cell_seq",
                "neighb_cell_structured_seq")


def _need_cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def make_gpu(scene, fluid_arrays, bound_arrays, use_graph=True):
    from tichi_sph_gb300 import sph_config, Fluid, Solver
    cfg = sph_config.load(*G.paths(scene))
    objs = []
    for uid, (cap, arrs) in enumerate(((cfg.fluid_max_part_num[None], fluid_arrays),
                                       (cfg.bound_max_part_num[None], bound_arrays))):
        o = Fluid(cap, cfg, uid, device="cuda")
        n = len(arrs["pos"])
        o.part_num[None] = n
        for k, v in arrs.items():
            getattr(o, k)[:n] = torch.as_tensor(np.asarray(v, dtype=np.float32), device="cuda").reshape(
                getattr(o, k)[:n].shape)
        objs.append(o)
    s = Solver(cfg, objs[0], objs[1], fbm=scene in G.FBM_SCENES, use_graph=use_graph,
               wcsph=scene in G.WC_SCENES)
    return cfg, objs[0], objs[1], s


def _substep_oracle(scene, ofl, obd, p, st, gold):
    """One oracle substep with the scene's optional blocks; returns the
    particle-to-grid map's node velocities for WC scenes (else None)."""
    wc = scene in G.WC_SCENES
    mg = G.map_grid(gold) if wc else None
    O.run_substep(ofl, obd, p, st, fbm=scene in G.FBM_SCENES, wc=wc, map_grid=mg)
    return mg["vel"] if wc else None


def _check_map(scene, tag, cfg, solver, ref):
    from tichi_sph_gb300.sph_obj import Grid
    grid = Grid(cfg, device="cuda")
    solver.map_velocity(grid)
    a = grid.vel.cpu().numpy().astype(np.float64)
    assert a.shape == ref.shape, (scene, a.shape, ref.shape)
    err = float(np.abs(a - ref).max()) / max(float(np.abs(ref).max()), 1e-30)
    assert err <= 1e-5, "%s %s grid velocity rel err %.3g" % (scene, tag, err)


def make_oracle(scene, fluid_arrays, bound_arrays):
    p = O.Params.from_files(*G.paths(scene), taichi_f32=True)
    f64 = lambda d: {k: np.asarray(v, dtype=np.float32).astype(np.float64) for k, v in d.items()}
    fl, bd = O.sets_from_arrays(p, f64(fluid_arrays), f64(bound_arrays))
    return p, fl, bd


def compare(scene, tag, gpu_set, ora_set, fields, tol_scale=1.0, dens_scale=None, fbm_dt=None):
    n = ora_set.n
    worst = {}
    vmax = float(np.abs(np.asarray(ora_set.vel_adv)).max(initial=0.0))
    for f in fields:
        a = getattr(gpu_set, f)[:n].detach().cpu().numpy().astype(np.float64)
        b = np.asarray(getattr(ora_set, f), dtype=np.float64).reshape(a.shape)
        if f in EXACT:
            np.testing.assert_array_equal(a, b, err_msg="%s %s %s" % (scene, tag, f))
            continue
        scale = float(np.abs(b).max(initial=0.0))
        if f == "psi_adv" and dens_scale is not None:
            scale = max(scale, dens_scale)
        if fbm_dt is not None:
            if f in ("acce_adv", "acce"):
                scale = max(scale, vmax / fbm_dt)
            elif f == "drift_vel":
                scale = max(scale, vmax)
            elif f == "volume_frac_tmp":
                scale = max(scale, float(np.abs(ora_set.volume_frac).max(initial=0.0)))
        err = float(np.abs(a - b).max(initial=0.0)) / max(scale, 1e-30)
        worst[f] = err
        assert err <= TOL_ONE_STEP[f] * tol_scale, "%s %s %s rel err %.3g > %.3g (scale %.3g)" % (
            scene, tag, f, err, TOL_ONE_STEP[f] * tol_scale, scale)
    return worst


def _fluid_fields(scene, p):
    fields = ["pos", "vel", "vel_adv", "acce_adv", "mass", "rest_density", "W", "sph_density",
              "sph_compression", "psi_adv", "alpha", "alpha_1", "alpha_2"] + list(EXACT)
    if p.surface_tension_gamma != 0:
        fields.append("normal")
    if scene in G.FBM_SCENES:
        fields += ["volume_frac", "volume_frac_tmp", "drift_vel", "fbm_zeta", "acce"]
    if scene in G.WC_SCENES:
        fields.append("pressure")
    return fields


@pytest.mark.parametrize("use_graph", [True, False], ids=["graph", "hostloop"])
@pytest.mark.parametrize("scene", G.SCENES)
def test_one_step_from_reference_states(scene, use_graph):
    """Each golden step k, started from the reference-run state after step k-1."""
    _need_cuda()
    init, gold = G.load(scene)
    for step in range(G.n_steps(gold)):
        if step == 0:
            fa, ba = G.init_arrays(init, "fluid"), G.init_arrays(init, "bound")
            t0, c0 = 0.0, 0.0
        else:
            pre = "s%d_" % (step - 1)
            fa = {k: gold[pre + "fluid_" + k] for k in G.STATE_IN}
            ba = {k: gold[pre + "bound_" + k] for k in G.STATE_IN}
            t0, c0 = float(gold[pre + "time_count"]), float(gold[pre + "compression"])
        cfg, fl, bd, solver = make_gpu(scene, fa, ba, use_graph)
        p, ofl, obd = make_oracle(scene, fa, ba)
        solver.set_state(time_count=t0, compression=c0)
        ofl.compression = c0
        st = O.Stats()
        st.time_count = t0
        solver.substep()
        gs = solver.stats()
        gref = _substep_oracle(scene, ofl, obd, p, st, gold)
        if gref is not None:
            _check_map(scene, "step%d" % step, cfg, solver, gref)
        assert gs["div_iter"] == st.div_iter and gs["incom_iter"] == st.incom_iter, (scene, step, gs, vars(st))
        assert gs["dt"] == pytest.approx(st.dt, rel=1e-6)
        if scene in G.FBM_SCENES:
            assert gs["fbm_passes"] == st.fbm_passes
        dens = float(np.abs(ofl.sph_density).max(initial=0.0))
        fdt = st.dt if scene in G.FBM_SCENES else None
        compare(scene, "step%d fluid" % step, fl, ofl, _fluid_fields(scene, p), dens_scale=dens, fbm_dt=fdt)
        compare(scene, "step%d bound" % step, bd, obd, BOUND_FIELDS)
        assert gs["compression"] == pytest.approx(ofl.compression, rel=1e-3, abs=1e-6)
        assert gs["kinetic_energy"] == pytest.approx(ofl.statistics_kinetic_energy, rel=1e-5)
        assert gs["potential_energy"] == pytest.approx(ofl.statistics_gravity_potential_energy, rel=1e-5)
        solver.close()


@pytest.mark.parametrize("scene", G.SCENES)
def test_trajectory_against_oracle(scene):
    """All golden steps chained on the GPU vs the oracle chained from the same
    f32 initial state: identical iteration counts, fields within 10x the
    one-step tolerance."""
    _need_cuda()
    init, gold = G.load(scene)
    fa, ba = G.init_arrays(init, "fluid"), G.init_arrays(init, "bound")
    cfg, fl, bd, solver = make_gpu(scene, fa, ba)
    p, ofl, obd = make_oracle(scene, fa, ba)
    st = O.Stats()
    for step in range(G.n_steps(gold)):
        solver.substep()
        gs = solver.stats()
        _substep_oracle(scene, ofl, obd, p, st, gold)
        assert gs["div_iter"] == st.div_iter and gs["incom_iter"] == st.incom_iter
        assert gs["time_count"] == pytest.approx(st.time_count, rel=1e-6)
        dens = float(np.abs(ofl.sph_density).max(initial=0.0))
        fdt = st.dt if scene in G.FBM_SCENES else None
        compare(scene, "traj%d" % step, fl, ofl, _fluid_fields(scene, p), tol_scale=10.0, dens_scale=dens,
                fbm_dt=fdt)
    solver.close()


def _mix64(x):
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return x ^ (x >> np.uint64(31))


def _oracle_neighbours(p, obj, nobj, grid, uid_bits):
    """(count, hash) of the 0 < r < h neighbours among `nobj`, FP32 distances."""
    pr = grid.pairs(obj, nobj)
    xi = obj.pos[pr.i].astype(np.float32)
    xj = nobj.pos[pr.j].astype(np.float32)
    d = xi - xj
    r2 = np.sum(d * d, axis=1, dtype=np.float32)
    q = np.sqrt(r2).astype(np.float32) * np.float32(1.0 / np.float32(p.h))
    m = (r2 > 0) & (q < 1)
    ties = np.abs(q.astype(np.float64) - 1.0) < 1e-6
    cnt = np.bincount(pr.i[m], minlength=obj.n)
    with np.errstate(over="ignore"):
        hv = _mix64(np.uint64(uid_bits) | pr.j[m].astype(np.uint64))
        h = np.zeros(obj.n, dtype=np.uint64)
        np.add.at(h, pr.i[m], hv)
    tie_rows = np.zeros(obj.n, dtype=bool)
    tie_rows[pr.i[ties]] = True
    return cnt, h, tie_rows


@pytest.mark.parametrize("scene", G.SCENES)
def test_neighbor_sets_bit_exact(scene):
    """Per-particle neighbour sets (fluid and boundary) equal the reference's
    template-cell candidates filtered by FP32 q < 1; rows with a pair within
    1e-6 of q = 1 are excluded."""
    _need_cuda()
    init, gold = G.load(scene)
    pre = "s0_"
    fa = {k: gold[pre + "fluid_" + k] for k in G.STATE_IN}
    ba = {k: gold[pre + "bound_" + k] for k in G.STATE_IN}
    cfg, fl, bd, solver = make_gpu(scene, fa, ba)
    p, ofl, obd = make_oracle(scene, fa, ba)
    fc, fh, bc, bh = [t.cpu().numpy() for t in solver.neighbor_stats()]
    grid = O.Grid(p, [ofl, obd])
    for obj, cnt_gpu, hash_gpu in ((ofl, fc, fh), (obd, bc, bh)):
        cf, hf, tf = _oracle_neighbours(p, obj, ofl, grid, 0)
        cb, hb, tb = _oracle_neighbours(p, obj, obd, grid, 1 << 32)
        keep = ~(tf | tb)
        np.testing.assert_array_equal(cnt_gpu[keep, 0], cf[keep])
        np.testing.assert_array_equal(cnt_gpu[keep, 1], cb[keep])
        np.testing.assert_array_equal(hash_gpu[keep].view(np.uint64), (hf + hb)[keep])
    solver.close()


@pytest.mark.parametrize("tpp", [1, 2, 8])
@pytest.mark.parametrize("scene", ["dfsph3d", "vfsph2d", "edge2d"])
def test_threads_per_particle_settings(scene, tpp):
    """Every threads-per-particle setting of the list sweeps meets the one-step bar."""
    _need_cuda()
    init, gold = G.load(scene)
    fa, ba = G.init_arrays(init, "fluid"), G.init_arrays(init, "bound")
    cfg, fl, bd, solver = make_gpu(scene, fa, ba)
    solver.set_threads_per_particle(tpp)
    p, ofl, obd = make_oracle(scene, fa, ba)
    solver.substep()
    gs = solver.stats()
    st = O.run_substep(ofl, obd, p, O.Stats(), fbm=scene in G.FBM_SCENES)
    assert (gs["div_iter"], gs["incom_iter"]) == (st.div_iter, st.incom_iter)
    dens = float(np.abs(ofl.sph_density).max(initial=0.0))
    fdt = st.dt if scene in G.FBM_SCENES else None
    compare(scene, "tpp%d" % tpp, fl, ofl, _fluid_fields(scene, p), dens_scale=dens, fbm_dt=fdt)
    solver.close()


@pytest.mark.parametrize("scene", ["dfsph3d", "vfsph2d"])
def test_bitwise_deterministic(scene):
    """Same inputs, same settings: bit-identical state after several substeps
    (ordered cell slots, fixed neighbour order, fixed-order FP64 reductions)."""
    _need_cuda()
    init, gold = G.load(scene)
    fa, ba = G.init_arrays(init, "fluid"), G.init_arrays(init, "bound")
    outs = []
    for _ in range(2):
        cfg, fl, bd, solver = make_gpu(scene, fa, ba)
        for _ in range(3):
            solver.substep()
        st = solver.stats()
        outs.append((fl.pos.cpu().numpy().copy(), fl.vel.cpu().numpy().copy(),
                     fl.volume_frac.cpu().numpy().copy(), st["compression"], st["kinetic_energy"]))
        solver.close()
    a, b = outs
    for x, y in zip(a, b):
        np.testing.assert_array_equal(np.asarray(x), np.asarray(y))


def _make_gpu_cfg(cfg_d, scen_d, fluid_arrays, bound_arrays):
    from tichi_sph_gb300 import sph_config, Fluid, Solver
    cfg = sph_config.Config(cfg_d, scen_d)
    objs = []
    for uid, (cap, arrs) in enumerate(((cfg.fluid_max_part_num[None], fluid_arrays),
                                       (cfg.bound_max_part_num[None], bound_arrays))):
        o = Fluid(cap, cfg, uid, device="cuda")
        n = len(arrs["pos"])
        o.part_num[None] = n
        for k, v in arrs.items():
            getattr(o, k)[:n] = torch.as_tensor(np.asarray(v, dtype=np.float32), device="cuda").reshape(
                getattr(o, k)[:n].shape)
        objs.append(o)
    return cfg, objs[0], objs[1], Solver(cfg, objs[0], objs[1])


@pytest.mark.parametrize("iter_min,carried", [(0, 0.0), (0, 0.5), (1, 0.0)])
def test_iteration_floor_and_carried_compression(iter_min, carried):
    """solver_iter_threshold_min below 2 (the golden scenes all use 2): with 0
    a solve runs only while the compression carried over from the previous
    solve is above its tolerance (main.py:201), so its first iteration may or
    may not run; with 1 the first runs and later ones follow the tolerance.
    Three chained substeps of the dfsph3d scene, GPU vs oracle: identical
    iteration counts, fields within 10x the one-step tolerance."""
    _need_cuda()
    import json
    scene = "dfsph3d"
    cpath, spath = G.paths(scene)
    cfg_d, scen_d = json.load(open(cpath)), json.load(open(spath))
    cfg_d["solver_iter_threshold_min"] = iter_min
    init, _ = G.load(scene)
    fa, ba = G.init_arrays(init, "fluid"), G.init_arrays(init, "bound")
    cfg, fl, bd, solver = _make_gpu_cfg(cfg_d, scen_d, fa, ba)
    p = O.Params.from_config(cfg_d, scen_d, taichi_f32=True)
    f64 = lambda d: {k: np.asarray(v, dtype=np.float32).astype(np.float64) for k, v in d.items()}
    ofl, obd = O.sets_from_arrays(p, f64(fa), f64(ba))
    solver.set_state(time_count=0.0, compression=carried)
    ofl.compression = carried
    st = O.Stats()
    iters = []
    for step in range(3):
        solver.substep()
        gs = solver.stats()
        O.run_substep(ofl, obd, p, st)
        assert (gs["div_iter"], gs["incom_iter"]) == (st.div_iter, st.incom_iter), (step, gs, vars(st))
        iters.append((st.div_iter, st.incom_iter))
        dens = float(np.abs(ofl.sph_density).max(initial=0.0))
        compare(scene, "floor%d step%d" % (iter_min, step), fl, ofl, _fluid_fields(scene, p), tol_scale=10.0,
                dens_scale=dens)
    solver.close()
    if iter_min == 0 and carried == 0.0:
        assert iters[0] == (0, 0)
    if iter_min == 0 and carried > 0.0:
        assert iters[0][0] >= 1
    if iter_min == 1:
        assert all(d >= 1 and i >= 1 for d, i in iters)


def _state_in(fl, bd):
    nf, nb = fl.part_num[None], bd.part_num[None]
    fa = {k: getattr(fl, k)[:nf].cpu().numpy().copy() for k in G.STATE_IN}
    ba = {k: getattr(bd, k)[:nb].cpu().numpy().copy() for k in G.STATE_IN}
    return fa, ba


def _step_outputs(fl, bd):
    nf, nb = fl.part_num[None], bd.part_num[None]
    out = {"fluid " + k: getattr(fl, k)[:nf].cpu().numpy().copy()
           for k in ("pos", "vel", "volume_frac", "W", "sph_density", "sph_compression", "psi_adv", "alpha")}
    out.update({"bound " + k: getattr(bd, k)[:nb].cpu().numpy().copy() for k in BOUND_FIELDS})
    return out


@pytest.mark.parametrize("scene", ["dfsph3d", "vfsph2d", "wcsph3d"])
def test_static_boundary_sums_kept_across_substeps(scene):
    """The boundary particles' sums over boundary neighbours are kept from the
    previous substep while the gather finds every boundary position and mass
    bitwise unchanged (the boundary adds them before its fluid terms).  A
    substep that kept them equals, bit for bit, the same substep in a fresh
    context, which computes them; so does a substep after the caller moved one
    boundary particle and changed another's mass, and one after such a change
    was first seen by a call that builds the grid alone (the neighbour stats)."""
    _need_cuda()
    init, _ = G.load(scene)
    cfg, fl, bd, solver = make_gpu(scene, G.init_arrays(init, "fluid"), G.init_arrays(init, "bound"))
    try:
        solver.substep()
        for case in ("unchanged", "moved", "moved, then the grid alone"):
            before = solver.stats()
            if case != "unchanged":
                bd.pos[0, 0] += 0.25 * float(cfg.part_size[1])
                bd.mass[1] *= 1.5
            if case == "moved, then the grid alone":
                solver.neighbor_stats()
            fa, ba = _state_in(fl, bd)
            solver.substep()
            got, got_st = _step_outputs(fl, bd), solver.stats()
            _, fl2, bd2, fresh = make_gpu(scene, fa, ba)
            fresh.set_state(time_count=before["time_count"], compression=before["compression"])
            fresh.substep()
            want, want_st = _step_outputs(fl2, bd2), fresh.stats()
            fresh.close()
            for k in want:
                np.testing.assert_array_equal(got[k], want[k], err_msg="%s %s %s" % (scene, case, k))
            for k in ("div_iter", "incom_iter", "compression", "kinetic_energy", "dt"):
                assert got_st[k] == want_st[k], (scene, case, k, got_st[k], want_st[k])
    finally:
        solver.close()
