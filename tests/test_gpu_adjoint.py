"""Discrete adjoint of n implicit steps (tf_adj_forward / tf_adj_backward).

The gradients of the apical shape loss with respect to per-element growth
rates and log Young's moduli are checked against central finite differences
of the GPU forward run (directional derivatives along seeded directions),
to 1e-6 relative.  The forward run itself is checked against the oracle's
Newton steps (node positions to 1e-8 relative).
"""
import numpy as np
import pytest

from oracle.oracle import Port
from tissuefolding_paperversion_gb300 import api, mesh

pytestmark = pytest.mark.gpu
TOL_GRAD = 1e-6


def _tissue(eta, seed=5):
    t = mesh.config_tiny(seed=seed, n=5, n_layers=2, eta=eta)
    rng = np.random.default_rng(seed + 100)
    rate = 1e-4 * (1.0 + 0.5 * rng.uniform(-1, 1, t.n_elems))   # 1/s, about 0.6 % per 60 s step
    logE = np.log(t.E)
    xy = t.pos.reshape(-1, 3)
    z_top = xy[t.node_placement == 1, 2].mean()
    c = xy[:, :2].mean(axis=0)
    params = np.array([c[0], c[1], 1.2 * z_top, 8.0])
    return t, rate, logE, params


def _solver(t):
    return api.Solver(t, newton_tol=1e-10, krylov_rtol=1e-12, krylov_max_iter=5000, deterministic=True)


def _loss(s, t, rate, logE, n, every, params):
    s.set_positions(t.pos)
    loss, saved = s.adjoint_forward(rate, logE, n, t.dt, every, params)
    return loss, saved


@pytest.mark.parametrize("eta,n,every", [(0.0, 4, 2), (100.0, 4, 2), (100.0, 5, 3), (100.0, 3, 1)])
def test_adjoint_matches_central_differences(eta, n, every):
    t, rate, logE, params = _tissue(eta)
    rng = np.random.default_rng(7)
    with _solver(t) as s:
        loss0, saved = _loss(s, t, rate, logE, n, every, params)
        gr, ge = s.adjoint_backward(saved)
        saved.free()
        assert np.all(np.isfinite(gr)) and np.all(np.isfinite(ge))
        assert np.abs(gr).max() > 0 and np.abs(ge).max() > 0
        for which in ("rate", "logE"):
            for _ in range(2):
                d = rng.standard_normal(t.n_elems)
                if which == "rate":
                    h = 1e-3 * np.abs(rate).mean()
                    lp, sp = _loss(s, t, rate + h * d, logE, n, every, params)
                    lm, sm = _loss(s, t, rate - h * d, logE, n, every, params)
                    adj = gr @ d
                else:
                    h = 1e-4
                    lp, sp = _loss(s, t, rate, logE + h * d, n, every, params)
                    lm, sm = _loss(s, t, rate, logE - h * d, n, every, params)
                    adj = ge @ d
                sp.free()
                sm.free()
                fd = (lp - lm) / (2 * h)
                assert abs(adj - fd) <= TOL_GRAD * abs(fd), (which, adj, fd)


def test_adjoint_matches_central_differences_32_directions():
    """32 seeded directions (16 along the growth rates, 16 along log E) on a
    3,200-prism sheet of the 320k-prism sheet's kind (log-normal E, internal
    viscosity 100, Gaussian growth bump), 20 steps, checkpoints every 5,
    multigrid solves.  Fourth-order central differences at h = 1e-2 (rates:
    1e-2 x the largest rate): a converged forward run is a function of its
    parameters only to ~1e-12 in the positions (Newton stops at |du| <=
    1e-11), which 2-point differences at h = 1e-6 amplify to ~1e-4 of the
    derivative along log E; at h = 1e-2 that noise is ~1e-8 and the
    truncation O(h^4)."""
    t = mesh.config_large(seed=7, cells=20)
    xy = t.pos.reshape(-1, 3)[:, :2]
    c = 0.5 * (xy.min(axis=0) + xy.max(axis=0))
    params = np.array([c[0], c[1], 5.0, 40.0])
    rate = t.rates.reshape(-1, 3)[:, 0].copy()
    logE = np.log(t.E)
    n, every, h = 20, 5, 1e-2
    rng = np.random.default_rng(4321)
    with api.Solver(t, newton_tol=1e-11, krylov_rtol=1e-13, deterministic=True, precond=2) as s:
        _, saved = _loss(s, t, rate, logE, n, every, params)
        gr, ge = s.adjoint_backward(saved)
        saved.free()

        def lossf(r, e):
            lv, sp = _loss(s, t, r, e, n, every, params)
            sp.free()
            return lv

        errs = []
        for k in range(32):
            d = rng.standard_normal(t.n_elems)
            if k % 2 == 0:
                hr = h * np.abs(rate).max()
                f = lambda a: lossf(rate + a * hr * d, logE)
                scale, adj = hr, gr @ d
            else:
                f = lambda a: lossf(rate, logE + a * h * d)
                scale, adj = h, ge @ d
            fd = (-f(2) + 8 * f(1) - 8 * f(-1) + f(-2)) / (12 * scale)
            errs.append(abs(adj - fd) / abs(fd))
    assert max(errs) <= TOL_GRAD, errs


def test_adjoint_gradient_is_independent_of_checkpoint_spacing():
    t, rate, logE, params = _tissue(100.0, seed=9)
    out = []
    with _solver(t) as s:
        for every in (1, 2, 5):
            _, saved = _loss(s, t, rate, logE, 5, every, params)
            out.append(s.adjoint_backward(saved))
            saved.free()
    for gr, ge in out[1:]:
        np.testing.assert_allclose(gr, out[0][0], rtol=1e-9, atol=1e-9 * np.abs(out[0][0]).max())
        np.testing.assert_allclose(ge, out[0][1], rtol=1e-9, atol=1e-9 * np.abs(out[0][1]).max())


def test_adjoint_forward_matches_oracle_steps():
    t, rate, logE, params = _tissue(100.0, seed=11)
    n = 3
    t.E = np.exp(logE)
    rates3 = np.zeros((t.n_elems, 3))
    rates3[:, 0] = rate
    rates3[:, 1] = rate
    p = Port(t)
    for _ in range(n):
        p.step(t.dt, rates3.reshape(-1))
    ref = p.positions()
    with _solver(t) as s:
        loss, saved = _loss(s, t, rate, logE, n, 2, params)
        got = s.positions()
        saved.free()
    scale = np.abs(ref).max()
    assert np.abs(got - ref).max() / scale <= 1e-8
    x = ref.reshape(-1, 3)[t.node_placement == 1]
    f = params[2] * np.exp(-((x[:, 0] - params[0]) ** 2 + (x[:, 1] - params[1]) ** 2) / (2 * params[3] ** 2))
    assert abs(loss - np.sum((x[:, 2] - f) ** 2)) <= 1e-7 * max(1.0, loss)


def test_adjoint_rejects_bad_arguments():
    t, rate, logE, params = _tissue(0.0)
    with _solver(t) as s:
        with pytest.raises(api.TfError):
            s.adjoint_forward(rate, logE, 0, t.dt, 1, params)
        with pytest.raises(api.TfError):
            s.adjoint_forward(rate, logE, 2, t.dt, 0, params)
        bad = params.copy()
        bad[3] = 0.0
        with pytest.raises(api.TfError):
            s.adjoint_forward(rate, logE, 2, t.dt, 1, bad)


def _oracle_loss(t, rate, logE, n, params):
    """Loss after n steps of the oracle's Newton solver (direct solves)."""
    t2 = mesh.Tissue(**{**t.__dict__, "E": np.exp(logE)})
    rates3 = np.zeros((t.n_elems, 3))
    rates3[:, 0] = rate
    rates3[:, 1] = rate
    p = Port(t2)
    for _ in range(n):
        p.step(t.dt, rates3.reshape(-1))
    x = p.positions().reshape(-1, 3)[t.node_placement == 1]
    f = params[2] * np.exp(-((x[:, 0] - params[0]) ** 2 + (x[:, 1] - params[1]) ** 2) / (2 * params[3] ** 2))
    return float(np.sum((x[:, 2] - f) ** 2))


@pytest.mark.parametrize("eta", [0.0, 100.0])
def test_adjoint_matches_differences_of_the_oracle_solver(eta):
    """The GPU adjoint against central differences of the CPU oracle's own
    Newton steps (the reference's algorithm with direct solves)."""
    t, rate, logE, params = _tissue(eta, seed=21)
    n = 3
    with _solver(t) as s:
        _, saved = _loss(s, t, rate, logE, n, 1, params)
        gr, ge = s.adjoint_backward(saved)
        saved.free()
    rng = np.random.default_rng(23)
    for which in ("rate", "logE"):
        d = rng.standard_normal(t.n_elems)
        if which == "rate":
            h = 1e-3 * np.abs(rate).mean()
            fd = (_oracle_loss(t, rate + h * d, logE, n, params) - _oracle_loss(t, rate - h * d, logE, n, params)) / (2 * h)
            adj = gr @ d
        else:
            h = 1e-4
            fd = (_oracle_loss(t, rate, logE + h * d, n, params) - _oracle_loss(t, rate, logE - h * d, n, params)) / (2 * h)
            adj = ge @ d
        assert abs(adj - fd) <= TOL_GRAD * abs(fd), (which, adj, fd)
