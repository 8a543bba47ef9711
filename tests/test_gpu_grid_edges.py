"""Neighbour sets on grid shapes where the reference's linear cell codes alias,
and the measurement entry points (needs a GPU).

The density sweep's candidate scan skips template rows and cells whose
geometry lies farther than h.  That is exact only when no template row can
alias another: with nx <= 2r (or ny <= 2r in 3D) the reference's template loop
(sph.py:52-60) reaches one cell through two offsets and counts its particles
twice, and the scan must then visit every candidate.  Seeded random clouds
that spill past the grid on every side (so some particles wrap into other rows
or have no valid code) are checked, per particle, against the oracle's template
candidates filtered by FP32 q < 1: counts and order-independent hashes of the
fluid and the boundary neighbour sets, rows with a pair within 1e-6 of q = 1
excluded.
"""
import numpy as np
import pytest
import torch

from oracle import sph_oracle as O

pytestmark = pytest.mark.gpu

H = 0.02


def _need_cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _scene(dim, nx_cells):
    from tichi_sph_gb300 import workloads
    cfg = workloads._config()
    span = [nx_cells * H - 0.25 * H] + [0.1] * (dim - 1)
    scen = {
        "sim_env": {"global_part_size": H / 2, "global_dynamic_viscosity": 0.01, "sim_dim": dim,
                    "sim_space_lb": [0.0] * dim, "sim_space_rt": span, "gravity": [0.0] * dim,
                    "phase_num": 1, "phase_rest_density": [1000], "phase_color_hex": ["0x6F7DBC"]},
        "fluid": {"max_part_num": 600, "objs": []},
        "bound": {"max_part_num": 200, "objs": []},
    }
    return cfg, scen, span


def _cloud(rng, n, dim, span):
    lo = -0.6 * H
    hi = np.asarray(span) + 0.6 * H
    return rng.uniform(lo, hi, size=(n, dim)).astype(np.float32)


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("nx_cells", [2, 3])
def test_neighbour_sets_on_narrow_grids(dim, nx_cells):
    _need_cuda()
    from tests.test_gpu_parity import _oracle_neighbours
    from tichi_sph_gb300 import Fluid, Solver, sph_config
    cfg_d, scen, span = _scene(dim, nx_cells)
    cfg = sph_config.Config(cfg_d, scen)
    assert int(cfg.neighb_grid_size[None][0]) == nx_cells
    rng = np.random.default_rng(100 * dim + nx_cells)
    pos = {"fluid": _cloud(rng, 600, dim, span), "bound": _cloud(rng, 200, dim, span)}
    sets = []
    for uid, name in enumerate(("fluid", "bound")):
        o = Fluid(len(pos[name]), cfg, uid, device="cuda")
        o.part_num[None] = len(pos[name])
        o.pos[:len(pos[name])] = torch.as_tensor(pos[name], device="cuda")
        o.mass[:len(pos[name])] = 1.0
        o.rest_density[:len(pos[name])] = 1000.0
        o.rest_volume[:len(pos[name])] = 1e-3
        o.volume_frac[:len(pos[name]), 0] = 1.0
        sets.append(o)
    solver = Solver(cfg, sets[0], sets[1])
    fc, fh, bc, bh = [t.cpu().numpy() for t in solver.neighbor_stats()]
    solver.close()
    p = O.Params.from_config(cfg_d, scen, taichi_f32=True)
    arr = lambda x: {"pos": x.astype(np.float64)}
    ofl, obd = O.sets_from_arrays(p, arr(pos["fluid"]), arr(pos["bound"]))
    grid = O.Grid(p, [ofl, obd])
    doubled = 0
    for obj, cnt_gpu, hash_gpu in ((ofl, fc, fh), (obd, bc, bh)):
        cf, hf, tf = _oracle_neighbours(p, obj, ofl, grid, 0)
        cb, hb, tb = _oracle_neighbours(p, obj, obd, grid, 1 << 32)
        keep = ~(tf | tb)
        assert keep.mean() > 0.95
        np.testing.assert_array_equal(cnt_gpu[keep, 0], cf[keep])
        np.testing.assert_array_equal(cnt_gpu[keep, 1], cb[keep])
        np.testing.assert_array_equal(hash_gpu[keep].view(np.uint64), (hf + hb)[keep])
        pr = grid.pairs(obj, ofl)
        doubled += len(pr.i) - len(set(zip(pr.i.tolist(), pr.j.tolist())))
    # the aliasing case really revisits cells; the other does not
    assert (doubled > 0) == (nx_cells == 2)


@pytest.mark.parametrize("nx_cells", [2, 3])
def test_candidate_counts(nx_cells):
    """tsph_candidate_stats: without skipping (aliasing rows) the scan visits
    exactly the reference template's candidates; with skipping, a subset of
    them that still holds every pair within h."""
    _need_cuda()
    from tests.test_gpu_parity import _oracle_neighbours
    from tichi_sph_gb300 import Fluid, Solver, sph_config
    dim = 3
    cfg_d, scen, span = _scene(dim, nx_cells)
    cfg = sph_config.Config(cfg_d, scen)
    rng = np.random.default_rng(7 + nx_cells)
    pos = {"fluid": _cloud(rng, 600, dim, span), "bound": _cloud(rng, 200, dim, span)}
    sets = []
    for uid, name in enumerate(("fluid", "bound")):
        o = Fluid(len(pos[name]), cfg, uid, device="cuda")
        o.part_num[None] = len(pos[name])
        o.pos[:len(pos[name])] = torch.as_tensor(pos[name], device="cuda")
        o.mass[:len(pos[name])] = 1.0
        o.rest_volume[:len(pos[name])] = 1e-3
        sets.append(o)
    solver = Solver(cfg, sets[0], sets[1])
    cf, cb = [t.cpu().numpy() for t in solver.candidate_stats()]
    solver.close()
    p = O.Params.from_config(cfg_d, scen, taichi_f32=True)
    arr = lambda x: {"pos": x.astype(np.float64)}
    ofl, obd = O.sets_from_arrays(p, arr(pos["fluid"]), arr(pos["bound"]))
    grid = O.Grid(p, [ofl, obd])
    for obj, cnt in ((ofl, cf), (obd, cb)):
        for col, nobj, bits in ((0, ofl, 0), (1, obd, 1 << 32)):
            tmpl = np.bincount(grid.pairs(obj, nobj).i, minlength=obj.n)
            pairs, _, _ = _oracle_neighbours(p, obj, nobj, grid, bits)
            if nx_cells == 2:
                np.testing.assert_array_equal(cnt[:, col], tmpl)
            else:
                assert (cnt[:, col] <= tmpl).all() and (cnt[:, col] >= pairs).all()
                assert cnt[:, col].sum() < tmpl.sum()


def test_fp32_fma_peak_is_plausible():
    _need_cuda()
    from tichi_sph_gb300.sph import fp32_fma_peak
    tf = fp32_fma_peak()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    # 128 FP32 lanes per SM, two operations per FMA, 0.5 - 3.5 GHz
    assert sms * 128 * 2 * 0.5e9 / 1e12 < tf < sms * 128 * 2 * 3.5e9 / 1e12, tf
