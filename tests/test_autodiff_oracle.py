"""Pins the FP64 autodiff oracle (CPU only).

* its forward substep equals the golden-pinned numpy oracle (``sph_step``);
* its gradients (torch.autograd) equal FP64 central finite differences;
* the hand-derived reverse pass -- the formulas the CUDA adjoint kernels
  implement -- equals torch.autograd to rounding.
"""
import numpy as np
import pytest
import torch

from oracle import sph_autodiff as A
from oracle import sph_oracle as O


def small_scene(nx=6, ny=6, nz=6, fixed_iters=2, relax=1.0, gamma=0.0):
    """The differentiable workload at a small size, as (params, numpy sets, autodiff scene, x0, v0, target)."""
    from tichi_sph_gb300 import sph_config, workloads
    from tichi_sph_gb300.simulation import Simulation
    c, s, vel, target = workloads.diff_block(nx=nx, ny=ny, nz=nz, fixed_iters=fixed_iters, relax=relax, gamma=gamma)
    cfg = sph_config.Config(c, s)
    sim = Simulation(cfg, device="cpu")
    sim.init_scenario()
    nf, nb = sim.fluid.part_num[None], sim.bound.part_num[None]
    keys = ["pos", "vel", "mass", "rest_volume", "rest_density", "volume_frac"]
    fa = {k: getattr(sim.fluid, k)[:nf].numpy().astype(np.float64) for k in keys}
    ba = {k: getattr(sim.bound, k)[:nb].numpy().astype(np.float64) for k in keys}
    fa["vel"] = vel(nf).astype(np.float64)
    p = O.Params.from_config(c, s, taichi_f32=True)
    dt = float(np.float32(np.float32(p.part_size) / np.float32(p.cs)))
    sc = A.Scene(3, p.h, p.sig, fa["mass"], fa["rest_density"], ba["pos"], ba["mass"], p.gravity, dt,
                 iters=(p.iter_min, p.iter_min), tol=(p.divergence_threshold, p.compression_threshold),
                 iter_max=p.iter_max, gamma=p.surface_tension_gamma, lb=p.lb)
    return p, fa, ba, sc, torch.as_tensor(fa["pos"]), torch.as_tensor(fa["vel"]), torch.as_tensor(target)


GAMMAS = [0.0, 0.07]   # without and with surface tension (the coefficient of the two-phase workload)


@pytest.mark.parametrize("gamma", GAMMAS)
def test_forward_matches_numpy_oracle(gamma):
    p, fa, ba, sc, x0, v0, _ = small_scene(fixed_iters=None, gamma=gamma)
    fluid, bound = O.sets_from_arrays(p, fa, ba)
    st = O.Stats()
    O.run_substep(fluid, bound, p, st)
    assert abs(st.dt - sc.dt) < 1e-12 * sc.dt
    x1, v1, comp, (kd, kp) = A.substep(sc, x0, v0, torch.tensor(p.viscosity, dtype=A.T))
    assert (kd, kp) == (st.div_iter, st.incom_iter)
    np.testing.assert_allclose(v1.numpy(), fluid.vel, rtol=0, atol=1e-12 * max(1.0, np.abs(fluid.vel).max()))
    np.testing.assert_allclose(x1.numpy(), fluid.pos, rtol=0, atol=1e-13)
    # compression is a mean of small positive parts of cancelling sums: absolute bound
    assert abs(comp - fluid.compression) <= 1e-15


def _rollout(sc, x0, v0, mu, steps, record=False):
    x, v, comp = x0, v0, 0.0
    recs = []
    for _ in range(steps):
        r = {} if record else None
        x, v, comp, _ = A.substep(sc, x, v, mu, comp, iters=(2, 2), record=r)
        recs.append(r)
    return x, v, recs


def _loss(sc, x0, v0, mu, target, steps):
    x, _, _ = _rollout(sc, x0, v0, mu, steps)
    return A.loss_fn(sc, x, target)


def _autograd(sc, x0, v0, mu, target, steps):
    v = v0.clone().requires_grad_(True)
    m = mu.clone().requires_grad_(True)
    L = _loss(sc, x0, v, m, target, steps)
    L.backward()
    return v.grad, m.grad


@pytest.mark.parametrize("gamma", GAMMAS)
def test_autograd_matches_central_differences(gamma):
    _, _, _, sc, x0, v0, target = small_scene(gamma=gamma)
    mu = torch.tensor(0.01, dtype=A.T)
    steps = 3
    gv, gmu = _autograd(sc, x0, v0, mu, target, steps)
    h = 1e-6
    with torch.no_grad():
        fd_mu = (_loss(sc, x0, v0, mu + h, target, steps) - _loss(sc, x0, v0, mu - h, target, steps)) / (2 * h)
        d = torch.as_tensor(np.random.default_rng(7).standard_normal(tuple(v0.shape)))
        fd_v = (_loss(sc, x0, v0 + h * d, mu, target, steps) - _loss(sc, x0, v0 - h * d, mu, target, steps)) / (2 * h)
    assert abs(float(fd_mu) - float(gmu)) <= 1e-5 * abs(float(gmu))
    assert abs(float(fd_v) - float((gv * d).sum())) <= 1e-5 * abs(float(fd_v))


@pytest.mark.parametrize("gamma", GAMMAS)
def test_hand_adjoint_matches_autograd(gamma):
    _, _, _, sc, x0, v0, target = small_scene(gamma=gamma)
    mu = torch.tensor(0.01, dtype=A.T)
    steps = 3
    gv_ref, gmu_ref = _autograd(sc, x0, v0, mu, target, steps)
    with torch.no_grad():
        xT, _, recs = _rollout(sc, x0, v0, mu, steps, record=True)
    xr = xT.clone().requires_grad_(True)
    m = sc.mass
    Lc = ((((m[:, None] * xr).sum(0) / m.sum()) - target) ** 2).sum()
    gx, = torch.autograd.grad(Lc, xr)
    rho, top = A.final_density(sc, xT)
    e = (rho - sc.rest_density) / sc.rest_density
    gx = gx + A.adjoint_final_density(sc, top, xT, 0.2 * e / sc.rest_density / len(e))
    gv = torch.zeros_like(gx)
    gmu = 0.0
    for r in reversed(recs):
        gx, gv, g = A.adjoint_substep(sc, r, mu, gx, gv)
        gmu += g
    assert float((gv - gv_ref).norm()) <= 1e-10 * float(gv_ref.norm())
    assert abs(gmu - float(gmu_ref)) <= 1e-10 * abs(float(gmu_ref))


@pytest.mark.parametrize("clamped", [False, True])
def test_hand_adjoint_clamps(clamped):
    """Both clamps active: a block whose psi_adv clamps at 0 for some particles,
    and (clamped=True) an isolated pair just inside h whose alpha sums are
    positive but below the 1e-4 floor."""
    _, _, _, sc, x0, v0, target = small_scene(4, 4, 4)
    if clamped:
        x0 = x0.clone()
        x0[-1] = x0[-1] + torch.tensor([0.3, 0.3, 0.3], dtype=A.T)
        x0[-2] = x0[-1] + torch.tensor([sc.h * (1 - 1e-5), 0.0, 0.0], dtype=A.T)
    mu = torch.tensor(0.05, dtype=A.T)
    gv_ref, gmu_ref = _autograd(sc, x0, v0, mu, target, 2)
    with torch.no_grad():
        xT, _, recs = _rollout(sc, x0, v0, mu, 2, record=True)
        alpha = recs[0]["alpha"]
        s_any = any(bool((s <= 0).any()) for (_, _, s) in recs[0]["log_d"] + recs[0]["log_p"])
    assert s_any
    if clamped:
        raw = (recs[0]["a1"] ** 2).sum(1) / sc.mass + recs[0]["a2"]
        assert bool(((alpha == 1e-4) & (raw > 0)).any())
    xr = xT.clone().requires_grad_(True)
    m = sc.mass
    Lc = ((((m[:, None] * xr).sum(0) / m.sum()) - target) ** 2).sum()
    gx, = torch.autograd.grad(Lc, xr)
    rho, top = A.final_density(sc, xT)
    e = (rho - sc.rest_density) / sc.rest_density
    gx = gx + A.adjoint_final_density(sc, top, xT, 0.2 * e / sc.rest_density / len(e))
    gv = torch.zeros_like(gx)
    gmu = 0.0
    for r in reversed(recs):
        gx, gv, g = A.adjoint_substep(sc, r, mu, gx, gv)
        gmu += g
    assert float((gv - gv_ref).norm()) <= 1e-10 * float(gv_ref.norm())
    assert abs(gmu - float(gmu_ref)) <= 1e-10 * abs(float(gmu_ref))


def test_cell_candidates_equal_the_reference_template():
    """The surface tension's candidate pairs of the autodiff oracle (cells at
    most one apart per axis) are exactly the numpy oracle's template candidates
    (sph.py:156-160 over the reference's linear cell codes), self pairs aside,
    and they hold every pair within h."""
    p, fa, ba, sc, x0, _, _ = small_scene(gamma=0.07)
    fluid, bound = O.sets_from_arrays(p, fa, ba)
    grid = O.Grid(p, [fluid, bound])
    pr = grid.pairs(fluid, fluid)
    ref = {(int(i), int(j)) for i, j in zip(pr.i, pr.j) if i != j}
    ci, cj = A.cell_candidates(fa["pos"], p.lb, p.h)
    got = set(zip(ci.tolist(), cj.tolist()))
    assert got == ref
    fi, fj = A.pairs(fa["pos"], fa["pos"], p.h, True)
    assert set(zip(fi.tolist(), fj.tolist())) <= got
