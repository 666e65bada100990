"""The large benchmark configurations on the GPU against the CPU oracle.

* the 995,824-prism wing-disc-like ellipse (8 layers, apical layers stiffer):
  its first implicit step -- the oracle's residual of the GPU's converged
  state, the residual both sides compute there, sampled element tangents;
* the 256-instance batched sweep (1k-50k prisms each, rectangular or
  elliptical, 2-4 layers): two batched steps of all instances; every
  instance's converged state is an equilibrium of the oracle's physics, and
  a seeded subset runs the oracle's own Newton steps (sparse storage, the
  Pardiso stand-in solve) with identical Newton counts and positions within
  1e-8;
* the adjoint on a 3,200-prism sheet against central differences of the
  oracle's Newton steps, and on the full 320,000-prism sheet (50 steps,
  checkpoints every 10) against central differences of the GPU forward run.

Forces of nearly unstressed elements are compared at the force scale E h^2
(FP64 evaluation at coordinates ~1000 um carries strain noise ~1e-13 in any
implementation, the reference's included)."""
import numpy as np
import pytest

from oracle import sparse
from oracle.oracle import CLOSED, LITERAL, Port
from tissuefolding_paperversion_gb300 import api, mesh

pytestmark = pytest.mark.gpu
TOL_K = 1e-11
TOL_POS = 1e-8
TOL_GRAD = 1e-6


def _rel(a, b):
    s = np.abs(b).max()
    return np.abs(a - b).max() / (s if s > 0 else 1.0)


def _force_scale(t):
    p = t.pos.reshape(-1, 3)
    c = t.conn.reshape(-1, 6)
    return float(np.max(t.E)) * float(np.mean(np.sum((p[c[:, 1]] - p[c[:, 0]]) ** 2, axis=1)))


def test_wing_first_step_matches_the_oracle():
    t = mesh.config_wing(seed=0)
    assert t.n_elems > 990000
    with api.Solver(t) as s:
        s.set_growth_rates(t.rates)
        out = s.newton_step(t.dt, allow_not_converged=False)
        assert out["converged"] and out["dunorm"][-1] <= 1e-8
        assert out["krylov_total"] > 0
        pos = s.positions()
        Fg, _ = s.get_Fg()
        s.set_state(pos, t.pos, t.dt)
        s.assemble()
        g_gpu = s.residual()
        area = s.viscosity_surfaces()
        sample = np.sort(np.random.default_rng(3).choice(t.n_elems, 32, replace=False))
        got = [s.element_eval(int(e), 1) for e in sample]
    p = Port(t)
    p.set_Fg(Fg)
    p.set_viscosity_surfaces(area)
    g_cpu = p.residual(pos, t.pos, t.dt)
    fs = _force_scale(t)
    assert np.abs(g_gpu - g_cpu).max() <= 1e-11 * fs
    assert np.abs(g_cpu).max() <= 1e-8 * fs
    for e, r in zip(sample, got):
        ref = p.element_eval(pos, t.pos, t.dt, LITERAL, int(e), 1)
        for k in ("Ke", "Kv"):
            assert _rel(r[k], ref[k]) <= TOL_K, (e, k)
        for k in ("fe", "fv"):
            assert np.abs(r[k] - ref[k]).max() <= 1e-11 * fs, (e, k)


def test_batched_sweep_matches_the_oracle():
    n_inst, n_steps = 256, 2
    ts = [mesh.config_batch_instance(s) for s in range(n_inst)]
    dt = ts[0].dt
    with api.Batch(ts) as b:
        b.set_growth_rates()
        iters, pos = [], []
        for _ in range(n_steps):
            out = b.step(dt, allow_not_converged=False)
            assert out["converged"].all()
            iters.append(out["iters"].copy())
            pos.append([b.instance_positions(i).copy() for i in range(n_inst)])
    # every instance: the converged state of the last step is an equilibrium
    # of the oracle's physics (growth, viscosity surfaces of the step's start)
    worst = 0.0
    for i, t in enumerate(ts):
        p = Port(t)
        for _ in range(n_steps):
            p.grow(dt, t.rates)
        p.set_positions(pos[-2][i])
        p.update_viscosity_surfaces()
        g = p.residual(pos[-1][i], pos[-2][i], dt)
        worst = max(worst, float(np.abs(g).max()) / _force_scale(t))
        p.close()
    assert worst <= 1e-8, worst
    # a seeded subset: the oracle's own Newton steps
    sizes = np.array([t.n_elems for t in ts])
    small = list(np.argsort(sizes)[:4])
    rng = np.random.default_rng(44)
    mid = [int(i) for i in rng.choice(np.flatnonzero((sizes > 5000) & (sizes < 15000)), 2, replace=False)]
    for i in small + mid:
        t = ts[i]
        p = Port(t)
        solver = sparse.TransposedSolve(t.pos.reshape(-1, 3)[:, :2])
        for k in range(n_steps):
            r = sparse.newton_step(p, solver, dt, t.rates, mode=CLOSED)
            assert r["iters"] == iters[k][i], (i, k, r["iters"], iters[k][i])
            assert _rel(pos[k][i], p.positions()) <= TOL_POS, (i, k)
        p.close()


def _loss_params(t):
    xy = t.pos.reshape(-1, 3)
    c = 0.5 * (xy[:, :2].min(axis=0) + xy[:, :2].max(axis=0))
    return np.array([c[0], c[1], 5.0, 40.0])


def _oracle_loss(t, rate, logE, n, params):
    """Loss after n steps of the oracle's Newton loop (sparse storage, the
    Pardiso stand-in solve)."""
    t2 = mesh.Tissue(**{**t.__dict__, "E": np.exp(logE)})
    rates3 = np.zeros((t.n_elems, 3))
    rates3[:, 0] = rate
    rates3[:, 1] = rate
    p = Port(t2)
    solver = sparse.TransposedSolve(t.pos.reshape(-1, 3)[:, :2])
    for _ in range(n):
        sparse.newton_step(p, solver, t.dt, rates3.reshape(-1), mode=CLOSED)
    x = p.positions().reshape(-1, 3)[t.node_placement == 1]
    p.close()
    f = params[2] * np.exp(-((x[:, 0] - params[0]) ** 2 + (x[:, 1] - params[1]) ** 2) / (2 * params[3] ** 2))
    return float(np.sum((x[:, 2] - f) ** 2))


def test_adjoint_on_a_3200_prism_sheet_matches_differences_of_the_oracle():
    """The sheet of the 320k-prism configuration at 20 x 20 cells (4 layers,
    E log-normal, internal viscosity 100), 6 steps, checkpoints every 3;
    central differences of the oracle's Newton steps along one seeded
    direction per parameter set (h = 1e-3 of the largest rate, 1e-4 in
    log E: steps that balance the difference's truncation against the FP64
    rounding of the loss)."""
    t = mesh.config_large(seed=0, cells=20)
    n, every = 6, 3
    rate = t.rates.reshape(-1, 3)[:, 0].copy()
    logE = np.log(t.E)
    params = _loss_params(t)
    params[3] = 20.0
    with api.Solver(t, newton_tol=1e-10, krylov_rtol=1e-12, deterministic=True) as s:
        s.set_positions(t.pos)
        _, sv = s.adjoint_forward(rate, logE, n, t.dt, every, params)
        gr, ge = s.adjoint_backward(sv)
        sv.free()
    rng = np.random.default_rng(31)
    for which in ("rate", "logE"):
        d = rng.standard_normal(t.n_elems)
        if which == "rate":
            h = 1e-3 * np.abs(rate).max()
            lp = _oracle_loss(t, rate + h * d, logE, n, params)
            lm = _oracle_loss(t, rate - h * d, logE, n, params)
            adj = float(gr @ d)
        else:
            h = 1e-4
            lp = _oracle_loss(t, rate, logE + h * d, n, params)
            lm = _oracle_loss(t, rate, logE - h * d, n, params)
            adj = float(ge @ d)
        fd = (lp - lm) / (2 * h)
        assert abs(adj - fd) <= TOL_GRAD * abs(fd), (which, adj, fd)


def test_adjoint_at_full_size_matches_central_differences():
    """320,000 prisms, 50 steps of 60 s, checkpoints every 10: the gradient
    along one seeded direction per parameter set against central differences
    of the GPU forward run, every solve tight (h = 1e-3 of the largest rate,
    1e-4 in log E; at h = 1e-6 the FP64 rounding of the loss, ~1.6e7 over
    40,401 apical nodes, leaves the difference uncertain by ~2e-4)."""
    t = mesh.config_large(seed=0)
    n, every = 50, 10
    rate = t.rates.reshape(-1, 3)[:, 0].copy()
    logE = np.log(t.E)
    params = _loss_params(t)
    with api.Solver(t, newton_tol=1e-11, krylov_rtol=1e-13) as s:
        def loss(r, e):
            s.set_positions(t.pos)
            lv, sv = s.adjoint_forward(r, e, n, t.dt, every, params)
            sv.free()
            return lv
        s.set_positions(t.pos)
        _, sv = s.adjoint_forward(rate, logE, n, t.dt, every, params)
        gr, ge = s.adjoint_backward(sv)
        sv.free()
        rng = np.random.default_rng(1234)
        for which in ("rate", "logE"):
            d = rng.standard_normal(t.n_elems)
            if which == "rate":
                h = 1e-3 * np.abs(rate).max()
                fd = (loss(rate + h * d, logE) - loss(rate - h * d, logE)) / (2 * h)
                adj = float(gr @ d)
            else:
                h = 1e-4
                fd = (loss(rate, logE + h * d) - loss(rate, logE - h * d)) / (2 * h)
                adj = float(ge @ d)
            assert abs(adj - fd) <= TOL_GRAD * abs(fd), (which, adj, fd)
