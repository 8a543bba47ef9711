"""FP64 reference of the differentiable DFSPH substep.  TEST INFRASTRUCTURE ONLY.

The checker of the hand-written adjoint (``tsph_substep_adjoint``): only
``tests/`` and ``bench.py``'s checks may import it.  The reference has no
autodiff, so parity rests on mathematics instead of recorded vectors:

* :func:`substep` restates one DFSPH substep of the reference -- density and
  alpha (``sph.py:50-105``), the divergence solve (``main.py:199-214``),
  gravity + viscosity (``sph.py:108-129``) and the density solve
  (``main.py:221-234``), the position update (``sph.py:265-269``) -- in
  PyTorch float64 with the neighbour pairs of the substep fixed (found at the
  substep's start, 0 < r < h), so ``torch.autograd`` differentiates it exactly.
  Its values are pinned to the numpy oracle (``sph_oracle.sph_step``) by
  ``tests/test_autodiff_oracle.py``, and its gradients to central finite
  differences.
* :func:`adjoint_substep` is the hand-derived reverse pass, written pair by
  pair in the gather form the CUDA kernels use; the same tests pin it to
  autograd.

Differentiable inputs: positions, velocities and the dynamic viscosity mu.
Held constant: masses, rest densities, the boundary, the time step (a CFL
min() whose kink the checked configurations stay away from), the iteration
counts of the two Jacobi solves and the pair lists (the neighbour topology is
fixed per substep).  The clamps psi_adv = max(s, 0) and alpha = max(raw, 1e-4)
are differentiated one-sided (derivative 1 where the argument is above the
clamp, else 0).
"""
import math

import numpy as np
import torch

T = torch.float64


# ----------------------------------------------------------------------------- kernels
def w_q(q):
    """Cubic spline shape (``sph_util.py:16-25``), w(q)."""
    a = 6 * (q ** 3 - q ** 2) + 1
    b = 2 * (1 - q) ** 3
    return torch.where(q <= 0.5, a, torch.where(q < 1, b, torch.zeros_like(q)))


def dw_q(q):
    """w'(q) (``sph_util.py:28-37`` without the sigma/h factor)."""
    a = 6 * (3 * q ** 2 - 2 * q)
    b = -6 * (1 - q) ** 2
    return torch.where(q <= 0.5, a, torch.where(q < 1, b, torch.zeros_like(q)))


def ddw_q(q):
    """w''(q) (differentiating the spline once more)."""
    a = 6 * (6 * q - 2)
    b = 12 * (1 - q)
    return torch.where(q <= 0.5, a, torch.where(q < 1, b, torch.zeros_like(q)))


def c_q(q):
    """Cohesion spline shape (``sph_util.py:4-13`` without 32 / (pi h^3))."""
    p = (1 - q) ** 3 * q ** 3
    return torch.where(q <= 0.5, 2 * p - 1 / 64, torch.where(q < 1, p, torch.zeros_like(q)))


def dc_q(q):
    """d c_q / dq: 3 q^2 (1 - q)^2 (1 - 2 q), doubled below q = 1/2."""
    p = 3 * q ** 2 * (1 - q) ** 2 * (1 - 2 * q)
    return torch.where(q <= 0.5, 2 * p, torch.where(q < 1, p, torch.zeros_like(q)))


class Scene:
    """Constants of a differentiable DFSPH scene (one phase, static boundary)."""

    def __init__(self, dim, h, sig, mass, rest_density, bpos, bmass, gravity, dt, iters=(2, 2), tol=(1e-2, 1e-3),
                 iter_max=100, bvel=None, gamma=0.0, lb=None):
        self.dim = dim
        self.h = float(h)
        self.sig = float(sig)
        self.mass = torch.as_tensor(mass, dtype=T)
        self.rest_density = torch.as_tensor(rest_density, dtype=T)
        self.bpos = torch.as_tensor(bpos, dtype=T).reshape(-1, dim)
        self.bmass = torch.as_tensor(bmass, dtype=T)
        self.bvel = torch.zeros_like(self.bpos) if bvel is None else torch.as_tensor(bvel, dtype=T)
        self.gravity = torch.as_tensor(gravity, dtype=T)
        self.dt = float(dt)
        self.iter_min = int(iters[0]), int(iters[1])
        self.tol = float(tol[0]), float(tol[1])
        self.iter_max = int(iter_max)
        self.lap = 2.0 * (2 + dim)
        self.eps = 0.01 * self.h ** 2
        self.gamma = float(gamma)
        self.csig = 32.0 / math.pi / self.h ** 3
        # grid origin: the surface tension's curvature term runs over the
        # template cells' candidates (cell = h), not only pairs within h
        self.lb = None if lb is None else np.asarray(lb, dtype=np.float64)

    def W(self, r):
        return self.sig * w_q(r / self.h)

    def dW(self, r):
        return self.sig / self.h * dw_q(r / self.h)

    def ddW(self, r):
        return self.sig / self.h ** 2 * ddw_q(r / self.h)

    def C(self, r):
        return self.csig * c_q(r / self.h)

    def dC(self, r):
        return self.csig / self.h * dc_q(r / self.h)


# ----------------------------------------------------------------------------- topology
def pairs(x, y, h, same):
    """Index pairs (i, j) with 0 < |x_i - y_j| < h (both directions when `same`)."""
    from scipy.spatial import cKDTree
    xa = np.asarray(x, dtype=np.float64)
    ya = np.asarray(y, dtype=np.float64)
    if len(xa) == 0 or len(ya) == 0:
        return torch.zeros(0, dtype=torch.long), torch.zeros(0, dtype=torch.long)
    tx = cKDTree(xa)
    ty = tx if same else cKDTree(ya)
    lst = tx.query_ball_tree(ty, r=h * (1 + 1e-9))
    ii, jj = [], []
    for i, js in enumerate(lst):
        for j in js:
            ii.append(i)
            jj.append(j)
    ii = np.array(ii, dtype=np.int64)
    jj = np.array(jj, dtype=np.int64)
    r = np.linalg.norm(xa[ii] - ya[jj], axis=1) if len(ii) else np.zeros(0)
    keep = (r > 0) & (r < h)
    return torch.as_tensor(ii[keep]), torch.as_tensor(jj[keep])


def cell_candidates(x, lb, h):
    """Directed fluid-fluid pairs (i, j), i != j, whose cells (``int((x - lb)
    // h)`` in FP32, ``sph_util.py:65-67``) differ by at most one per axis: the
    3^dim template's candidates of ``sph.py:156-160`` for particles away from
    the grid's edges."""
    f32 = np.float32
    cell = np.floor((np.asarray(x, dtype=f32) - lb.astype(f32)) / f32(h)).astype(np.int64)
    d = np.abs(cell[:, None, :] - cell[None, :, :]).max(axis=2)
    ii, jj = np.nonzero(d <= 1)
    keep = ii != jj
    return torch.as_tensor(ii[keep]), torch.as_tensor(jj[keep])


class Topology:
    """Fluid-fluid pairs (directed, both ways) and fluid-boundary pairs of a
    substep; with surface tension on, also the template candidates (ci, cj)."""

    def __init__(self, sc, x):
        xd = x.detach().cpu().numpy()
        self.fi, self.fj = pairs(xd, xd, sc.h, True)
        self.bi, self.bj = pairs(xd, sc.bpos.numpy(), sc.h, False)
        if sc.gamma != 0.0:
            if sc.lb is None:
                raise ValueError("surface tension needs the grid origin (Scene lb)")
            ci, cj = cell_candidates(xd, sc.lb, sc.h)
            r = np.linalg.norm(xd[ci.numpy()] - xd[cj.numpy()], axis=1)
            keep = torch.as_tensor(r > 0)
            self.ci, self.cj = ci[keep], cj[keep]


def _sum(idx, vals, n):
    out = torch.zeros((n,) + tuple(vals.shape[1:]), dtype=vals.dtype)
    return out.index_add(0, idx, vals)


# ----------------------------------------------------------------------------- forward
def density_alpha(sc, top, x):
    """SPH_prepare_attr + alpha_1/alpha_2/alpha (sph.py:50-105) for DFSPH (X = mass)."""
    n = x.shape[0]
    m = sc.mass
    rf = x[top.fi] - x[top.fj]
    r = rf.norm(dim=1)
    rb = x[top.bi] - sc.bpos[top.bj]
    s = rb.norm(dim=1)
    rho = m * sc.W(torch.zeros(1, dtype=T)) + _sum(top.fi, m[top.fj] * sc.W(r), n) + _sum(top.bi, sc.bmass[top.bj] * sc.W(s), n)
    gf = (sc.dW(r) / r)[:, None] * rf
    gb = (sc.dW(s) / s)[:, None] * rb
    a1 = _sum(top.fi, m[top.fj][:, None] * gf, n) + _sum(top.bi, sc.bmass[top.bj][:, None] * gb, n)
    a2 = _sum(top.fi, (gf * gf).sum(1) * m[top.fj] ** 2 / m[top.fj], n)
    raw = (a1 * a1).sum(1) / m + a2
    alpha = torch.clamp(raw, min=1e-4)
    return rho, alpha, a1, a2


def solve_iteration(sc, top, x, u, psi, alpha):
    """IPPE_adv_psi_init / adv_psi / non_negative / update_vel_adv (sph.py:196-244)."""
    n = x.shape[0]
    m = sc.mass
    dt = sc.dt
    rf = x[top.fi] - x[top.fj]
    r = rf.norm(dim=1)
    gf = (sc.dW(r) / r)[:, None] * rf
    rb = x[top.bi] - sc.bpos[top.bj]
    s_ = rb.norm(dim=1)
    gb = (sc.dW(s_) / s_)[:, None] * rb
    div = _sum(top.fi, m[top.fj] * (gf * (u[top.fi] - u[top.fj])).sum(1), n) \
        + _sum(top.bi, sc.bmass[top.bj] * (gb * (u[top.bi] - sc.bvel[top.bj])).sum(1), n)
    s = psi - sc.rest_density + dt * div
    psi_adv = torch.clamp(s, min=0.0)
    comp = float((psi_adv / sc.rest_density).mean().detach()) if n else float("nan")
    kap = psi_adv / alpha
    f = _sum(top.fi, (kap[top.fi] * m[top.fj] + kap[top.fj] * m[top.fi])[:, None] * gf, n) \
        + _sum(top.bi, (kap[top.bi] * sc.bmass[top.bj])[:, None] * gb, n)
    u2 = u - f / (dt * m)[:, None]
    return u2, kap, s, comp


def viscosity_acc(sc, top, x, v, psi, mu):
    """SPH_advection_gravity_acc + viscosity_acc (sph.py:108-129), fluid-fluid."""
    n = x.shape[0]
    rf = x[top.fi] - x[top.fj]
    r2 = (rf * rf).sum(1)
    r = r2.sqrt()
    g = sc.dW(r) / r
    vr = ((v[top.fi] - v[top.fj]) * rf).sum(1)
    f = sc.lap * (sc.mass[top.fj] / psi[top.fj]) * g * vr / (sc.eps + r2)
    V = _sum(top.fi, f[:, None] * rf, n) / sc.rest_density[:, None]
    return sc.gravity[None, :] + mu * V


def surface_tension_acc(sc, top, x, psi):
    """SPH_advection_surface_tension_acc (sph.py:132-166), fluid-fluid, one
    phase (volume fraction 1 everywhere): normals n_i = h sum_j -(X_j / psi_j)
    g_ij r_ij, then a_i += sum_j 2 psi0_i / (psi_i + psi_j) (-gamma m_j C(r)
    r_ij / r + gamma (n_i - n_j)).  The second sum runs over every template
    candidate with r > 0, as the reference's loop does: the curvature term has
    no kernel weight, so candidates beyond h contribute to it (C = 0 there).
    Returns (acceleration, normals)."""
    n = x.shape[0]
    m = sc.mass
    fi, fj = top.fi, top.fj
    rf = x[fi] - x[fj]
    r = rf.norm(dim=1)
    g = sc.dW(r) / r
    nrm = sc.h * _sum(fi, (-(m[fj] / psi[fj]) * g)[:, None] * rf, n)
    ci, cj = top.ci, top.cj
    rc = x[ci] - x[cj]
    s = rc.norm(dim=1)
    c = 2 * sc.rest_density[ci] / (psi[ci] + psi[cj])
    coh = (-sc.gamma * m[cj] * sc.C(s) / s)[:, None] * rc
    cur = sc.gamma * (nrm[ci] - nrm[cj])
    return _sum(ci, c[:, None] * (coh + cur), n), nrm


def solve(sc, top, x, u, psi, alpha, kind, compression, fixed_iters=None):
    """The loop of main.py:199-214 / 221-234 (iteration count recorded)."""
    it, comp = 0, compression
    log = []
    while True:
        if fixed_iters is not None:
            if it >= fixed_iters:
                break
        elif not (it < sc.iter_min[kind] or comp > sc.tol[kind]):
            break
        u_in = u
        u, kap, s, comp = solve_iteration(sc, top, x, u, psi, alpha)
        log.append((u_in, kap, s))
        it += 1
        if fixed_iters is None and it > sc.iter_max:
            break
    return u, it, comp, log


def substep(sc, x, v, mu, compression=0.0, top=None, iters=None, record=None):
    """One DFSPH substep; returns (x', v', compression, iteration counts).
    `iters` = (k_div, k_dens) replays fixed counts; `record` (a dict) collects
    the intermediates the hand adjoint needs."""
    if top is None:
        top = Topology(sc, x)
    rho, alpha, a1, a2 = density_alpha(sc, top, x)
    psi = rho
    u, kd, compression, log_d = solve(sc, top, x, v, psi, alpha, 0, compression, None if iters is None else iters[0])
    vmid = u
    acc = viscosity_acc(sc, top, x, vmid, psi, mu)
    nrm = None
    if sc.gamma != 0.0:
        st, nrm = surface_tension_acc(sc, top, x, psi)
        acc = acc + st
    u = vmid + acc * sc.dt
    u, kp, compression, log_p = solve(sc, top, x, u, psi, alpha, 1, compression, None if iters is None else iters[1])
    x2 = x + u * sc.dt
    if record is not None:
        record.update(top=top, rho=rho, alpha=alpha, a1=a1, a2=a2, vmid=vmid, log_d=log_d, log_p=log_p, x=x,
                      nrm=nrm)
    return x2, u, compression, (kd, kp)


def final_density(sc, x, top=None):
    if top is None:
        top = Topology(sc, x)
    return density_alpha(sc, top, x)[0], top


def rollout(sc, x0, v0, mu, steps, iters=None):
    """`steps` substeps from (x0, v0); returns (x_T, v_T, per-step iteration counts)."""
    x, v, comp = x0, v0, 0.0
    counts = []
    for t in range(steps):
        x, v, comp, k = substep(sc, x, v, mu, comp, iters=None if iters is None else iters[t])
        counts.append(k)
    return x, v, counts


def loss_fn(sc, x, target, weight=0.1):
    """|CoM - target|^2 + weight * mean(((rho - rho0) / rho0)^2) at positions x."""
    m = sc.mass
    com = (m[:, None] * x).sum(0) / m.sum()
    rho, _ = final_density(sc, x)
    e = (rho - sc.rest_density) / sc.rest_density
    return ((com - target) ** 2).sum() + weight * (e * e).mean()


# ----------------------------------------------------------------------------- hand adjoint
def _pair_geom(sc, xi, xj):
    rv = xi - xj
    r2 = (rv * rv).sum(1)
    r = r2.sqrt()
    dW = sc.dW(r)
    g = dW / r
    G2 = (sc.ddW(r) - g) / r2   # g'(r) / r
    return rv, r, r2, g, G2, dW


def _dgrad(g, G2, rv, w):
    """d/dr_ij of (g(r) r_ij . w) as a vector: g w + G2 (r_ij . w) r_ij."""
    return g[:, None] * w + (G2 * (rv * w).sum(1))[:, None] * rv


def adjoint_iteration(sc, top, x, u, kap, s, alpha, lam_u2, lam_x, lam_psi, lam_alpha):
    """Reverse of one Jacobi iteration in the gather form of the CUDA sweeps.
    Returns lam_u (adjoint of the iteration's input velocities); adds into
    lam_x, lam_psi, lam_alpha."""
    n = x.shape[0]
    m = sc.mass
    dt = sc.dt
    fi, fj, bi, bj = top.fi, top.fj, top.bi, top.bj
    rv, r, r2, g, G2, _ = _pair_geom(sc, x[fi], x[fj])
    rb, rbn, rb2, gb, G2b, _ = _pair_geom(sc, x[bi], sc.bpos[bj])
    Xb = sc.bmass[bj]
    # sweep 1: lam_kappa and the position terms of the velocity update
    beta = lam_u2 / (dt * m)[:, None]
    db = beta[fi] - beta[fj]
    lam_k = -_sum(fi, m[fj] * g * (rv * db).sum(1), n) - _sum(bi, Xb * gb * (rb * beta[bi]).sum(1), n)
    cK = kap[fi] * m[fj] + kap[fj] * m[fi]
    lam_x -= _sum(fi, cK[:, None] * _dgrad(g, G2, rv, db), n)
    lam_x -= _sum(bi, (kap[bi] * Xb)[:, None] * _dgrad(gb, G2b, rb, beta[bi]), n)
    lam_s = torch.where(s > 0, lam_k / alpha, torch.zeros_like(lam_k))
    lam_alpha -= lam_k * kap / alpha
    lam_psi += lam_s
    # sweep 2: lam_u and the position terms of the divergence
    cS = lam_s[fi] * m[fj] + lam_s[fj] * m[fi]
    lam_u = lam_u2 + dt * _sum(fi, cS[:, None] * g[:, None] * rv, n) \
        + dt * _sum(bi, (lam_s[bi] * Xb * gb)[:, None] * rb, n)
    du = u[fi] - u[fj]
    lam_x += dt * _sum(fi, cS[:, None] * _dgrad(g, G2, rv, du), n)
    lam_x += dt * _sum(bi, (lam_s[bi] * Xb)[:, None] * _dgrad(gb, G2b, rb, u[bi] - sc.bvel[bj]), n)
    return lam_u


def adjoint_viscosity(sc, top, x, v, psi, mu, lam_a, lam_x, lam_psi):
    """Reverse of a = g + mu V(x, v, psi): returns (lam_v, dL/dmu); adds into lam_x, lam_psi."""
    n = x.shape[0]
    m = sc.mass
    fi, fj = top.fi, top.fj
    rv, r, r2, g, G2, _ = _pair_geom(sc, x[fi], x[fj])
    den = sc.eps + r2
    phi = g / den
    dphi = G2 / den - 2 * g / den ** 2     # phi'(r) / r
    vv = v[fi] - v[fj]
    vr = (vv * rv).sum(1)
    ci = mu * sc.lap * m[fj] / (sc.rest_density[fi] * psi[fj])   # coefficient of T_ij
    cj = mu * sc.lap * m[fi] / (sc.rest_density[fj] * psi[fi])   # coefficient of T_ji
    la_i, la_j = lam_a[fi], lam_a[fj]
    rli, rlj = (rv * la_i).sum(1), (rv * la_j).sum(1)
    lam_v = _sum(fi, ((ci * rli - cj * rlj) * phi)[:, None] * rv, n)
    lam_psi += _sum(fi, cj * phi * vr * rlj / psi[fi], n)
    lam_x += _sum(fi, ci[:, None] * (phi[:, None] * (rli[:, None] * vv + vr[:, None] * la_i)
                                     + (vr * rli * dphi)[:, None] * rv), n)
    lam_x -= _sum(fi, cj[:, None] * (phi[:, None] * (rlj[:, None] * vv + vr[:, None] * la_j)
                                     + (vr * rlj * dphi)[:, None] * rv), n)
    V = _sum(fi, (sc.lap * (m[fj] / psi[fj]) * phi * vr)[:, None] * rv, n) / sc.rest_density[:, None]
    gmu = float((lam_a * V).sum())
    return lam_v, gmu


def adjoint_surface_tension(sc, top, x, psi, nrm, lam_a, lam_x, lam_psi):
    """Reverse of :func:`surface_tension_acc` in two gather sweeps: adds into
    lam_x and lam_psi.  With c_ij = 2 psi0_i / (psi_i + psi_j) and B_ij =
    -gamma m_j C(r) r_ij / r + gamma (n_i - n_j), a_i = sum_j c_ij B_ij, so

      lam_n_i    = gamma sum_j (c_ij lam_a_i - c_ji lam_a_j),
      lam_psi_i -= sum_j (c_ij lam_a_i.B_ij + c_ji lam_a_j.B_ji) / (psi_i + psi_j),
      lam_x_i   += sum_j (k_ij D_C(lam_a_i) - k_ji D_C(lam_a_j)),  k_ij = -gamma m_j c_ij,
      D_C(w) = (C/r) w + ((C' - C/r) / r^2)(r_ij.w) r_ij (the cohesion's pair term);

    then the normals' reverse, sweep 2:

      lam_x_i   += h sum_j ((m_i / psi_i) D(lam_n_j) - (m_j / psi_j) D(lam_n_i)),
      lam_psi_i -= h (m_i / psi_i^2) sum_j g_ij r_ij.lam_n_j,

    D the pair gradient's derivative of :func:`_dgrad`."""
    n = x.shape[0]
    m = sc.mass
    gam = sc.gamma
    # sweep 1, over the template candidates: lam_n, the psi terms of c, the
    # cohesion's position terms
    ci, cj = top.ci, top.cj
    rc, s_, s2, _, _, _ = _pair_geom(sc, x[ci], x[cj])
    gC = sc.C(s_) / s_
    G2C = (sc.dC(s_) - gC) / s2
    s = psi[ci] + psi[cj]
    cij = 2 * sc.rest_density[ci] / s
    cji = 2 * sc.rest_density[cj] / s
    dn = nrm[ci] - nrm[cj]
    Bij = (-gam * m[cj] * gC)[:, None] * rc + gam * dn
    Bji = (gam * m[ci] * gC)[:, None] * rc - gam * dn
    la_i, la_j = lam_a[ci], lam_a[cj]
    lam_n = gam * _sum(ci, cij[:, None] * la_i - cji[:, None] * la_j, n)
    lam_psi -= _sum(ci, (cij * (la_i * Bij).sum(1) + cji * (la_j * Bji).sum(1)) / s, n)
    kij, kji = -gam * m[cj] * cij, -gam * m[ci] * cji
    lam_x += _sum(ci, kij[:, None] * _dgrad(gC, G2C, rc, la_i) - kji[:, None] * _dgrad(gC, G2C, rc, la_j), n)
    # sweep 2, over the pairs within h: the normals' reverse
    fi, fj = top.fi, top.fj
    rv, r, r2, g, G2, _ = _pair_geom(sc, x[fi], x[fj])
    ln_i, ln_j = lam_n[fi], lam_n[fj]
    lam_x += sc.h * _sum(fi, (m[fi] / psi[fi])[:, None] * _dgrad(g, G2, rv, ln_j)
                         - (m[fj] / psi[fj])[:, None] * _dgrad(g, G2, rv, ln_i), n)
    lam_psi -= sc.h * m / psi ** 2 * _sum(fi, g * (rv * ln_j).sum(1), n)


def adjoint_density_alpha(sc, top, x, a1, a2, lam_psi, lam_alpha, lam_x):
    """Reverse of density + alpha (sph.py:50-105): adds the position terms into lam_x."""
    n = x.shape[0]
    m = sc.mass
    fi, fj, bi, bj = top.fi, top.fj, top.bi, top.bj
    raw = (a1 * a1).sum(1) / m + a2
    on = (raw >= 1e-4).to(T)
    la1 = (lam_alpha * on * 2 / m)[:, None] * a1
    la2 = lam_alpha * on
    rv, r, r2, g, G2, dW = _pair_geom(sc, x[fi], x[fj])
    rb, rbn, rb2, gb, G2b, _ = _pair_geom(sc, x[bi], sc.bpos[bj])
    Xb = sc.bmass[bj]
    cR = lam_psi[fi] * m[fj] + lam_psi[fj] * m[fi]
    lam_x += _sum(fi, (cR * g)[:, None] * rv, n) + _sum(bi, (lam_psi[bi] * Xb * gb)[:, None] * rb, n)
    lam_x += _sum(fi, m[fj][:, None] * _dgrad(g, G2, rv, la1[fi]) - m[fi][:, None] * _dgrad(g, G2, rv, la1[fj]), n)
    lam_x += _sum(bi, Xb[:, None] * _dgrad(gb, G2b, rb, la1[bi]), n)
    c2 = la2[fi] * m[fj] ** 2 / m[fj] + la2[fj] * m[fi] ** 2 / m[fi]
    lam_x += _sum(fi, (c2 * 2 * g * sc.ddW(r))[:, None] * rv, n)


def adjoint_substep(sc, rec, mu, lam_x2, lam_v2):
    """Reverse of :func:`substep` from its record: (lam_x, lam_v, dL/dmu)."""
    x, top = rec["x"], rec["top"]
    psi, alpha = rec["rho"], rec["alpha"]
    dt = sc.dt
    lam_x = lam_x2.clone()
    lam_u = lam_v2 + dt * lam_x2
    lam_psi = torch.zeros_like(psi)
    lam_alpha = torch.zeros_like(psi)
    for (u, kap, s) in reversed(rec["log_p"]):
        lam_u = adjoint_iteration(sc, top, x, u, kap, s, alpha, lam_u, lam_x, lam_psi, lam_alpha)
    lam_a = lam_u * dt
    lam_vv, gmu = adjoint_viscosity(sc, top, x, rec["vmid"], psi, mu, lam_a, lam_x, lam_psi)
    if sc.gamma != 0.0:
        adjoint_surface_tension(sc, top, x, psi, rec["nrm"], lam_a, lam_x, lam_psi)
    lam_u = lam_u + lam_vv
    for (u, kap, s) in reversed(rec["log_d"]):
        lam_u = adjoint_iteration(sc, top, x, u, kap, s, alpha, lam_u, lam_x, lam_psi, lam_alpha)
    adjoint_density_alpha(sc, top, x, rec["a1"], rec["a2"], lam_psi, lam_alpha, lam_x)
    return lam_x, lam_u, gmu


def adjoint_final_density(sc, top, x, lam_rho):
    """Reverse of :func:`final_density`: dL/dx from dL/drho."""
    lam_x = torch.zeros_like(x)
    zero = torch.zeros_like(lam_rho)
    a1 = torch.zeros_like(x)
    adjoint_density_alpha(sc, top, x, a1, zero, lam_rho, zero, lam_x)
    return lam_x


# ----------------------------------------------------------------------------- scenes
def block_scene(nx, ny, nz, spacing=0.01, seed=5, v_std=0.1, rest_density=1000.0, dt=5e-4, iters=(2, 2),
                tol=(1e-2, 1e-3), floor=True):
    """A fluid block on a 3-layer floor of boundary particles (3D), as plain
    arrays: (Scene, x0, v0).  Lattice and masses follow the reference emitter's
    rules (rest_volume = spacing^dim, mass = rest_density * rest_volume)."""
    rng = np.random.default_rng(seed)
    sp = spacing
    g = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"), -1).reshape(-1, 3)
    x0 = (g * sp + 0.5 * sp).astype(np.float32).astype(np.float64)
    n = len(x0)
    v0 = (rng.standard_normal((n, 3)) * v_std).astype(np.float32).astype(np.float64)
    V = float(np.float32(sp ** 3))
    m = float(np.float32(rest_density * V))
    if floor:
        lx, lz = nx + 6, nz + 6
        gb = np.stack(np.meshgrid(np.arange(lx), np.arange(3), np.arange(lz), indexing="ij"), -1).reshape(-1, 3)
        bpos = ((gb - np.array([3, 3, 3])) * sp + 0.5 * sp).astype(np.float32).astype(np.float64)
    else:
        bpos = np.zeros((0, 3))
    h = float(np.float32(2 * sp))
    sig = float(np.float32(8 / math.pi / h ** 3))
    sc = Scene(3, h, sig, np.full(n, m), np.full(n, float(np.float32(rest_density))), bpos,
               np.full(len(bpos), m), [0.0, -9.81, 0.0], dt, iters=iters, tol=tol)
    return sc, torch.as_tensor(x0, dtype=T), torch.as_tensor(v0, dtype=T)
