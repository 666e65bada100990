"""Aggregation multigrid preconditioners: smoothed (tf_options.precond = 2)
and plain (3) aggregation.

The preconditioner changes how the Krylov solve gets to its tolerance, not
the system solved: Newton steps must still match the reference's golden
positions to 1e-8 with the same Newton iteration counts, solutions must
agree with the block-Jacobi solve to the Krylov tolerance, and the Krylov
iteration count must drop well below block-Jacobi's on sheets of a few
thousand nodes and more, and smoothing the prolongator must cut it below
plain aggregation's."""
import os

import numpy as np
import pytest

from tissuefolding_paperversion_gb300 import api, mesh

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
TOL_POS = 1e-8


def _steps(fixture, t, precond=2):
    f = np.load(os.path.join(GOLD, fixture + ".npz"))
    with api.Solver(t, precond=precond) as s:
        s.set_growth_rates(t.rates)
        for k in range(f["positions"].shape[0]):
            out = s.newton_step(t.dt, allow_not_converged=False)
            ref = f["positions"][k]
            pos = s.positions()
            assert np.abs(pos - ref).max() <= TOL_POS * np.abs(ref).max(), (k, np.abs(pos - ref).max())
            assert out["iters"] == f["iters"][k], (k, out["iters"])


@pytest.mark.parametrize("precond", [2, 3])
def test_multigrid_newton_steps_match_reference_small_config(precond):
    _steps("steps_small", mesh.config_small(seed=0), precond)


@pytest.mark.parametrize("precond", [2, 3])
@pytest.mark.parametrize("name,seed,eta", [("steps_tiny_elastic", 13, 0.0), ("steps_tiny_viscous", 14, 100.0)])
def test_multigrid_newton_steps_match_reference_tiny(name, seed, eta, precond):
    _steps(name, mesh.config_tiny(seed=seed, n=4, n_layers=2, eta=eta), precond)


@pytest.mark.parametrize("eta", [0.0, 100.0])
def test_multigrid_solution_matches_block_jacobi(eta):
    t = mesh.config_large(seed=3, cells=40)
    t.eta[:] = eta
    Fg = mesh.growth_Fg(t, seed=5, amp=0.01)
    uk, un = mesh.perturbed_state(t, seed=6, amp=0.05)
    out = {}
    for pc in (1, 2, 3):
        with api.Solver(t, precond=pc, krylov_rtol=1e-11) as s:
            s.set_Fg(Fg)
            s.set_positions(un)
            s.begin_step(t.dt)          # viscosity surfaces at the step's start shape
            s.set_state(uk, un, t.dt)
            s.assemble()
            r = s.solve()
            out[pc] = (s.delta_u(), r["iters"], r["relres"])
    du1, it1, rr1 = out[1]
    for pc in (2, 3):
        du2, it2, rr2 = out[pc]
        assert rr1 <= 1e-11 and rr2 <= 1e-11
        assert np.abs(du2 - du1).max() <= 1e-7 * np.abs(du1).max(), pc
        assert it2 * 4 <= it1, (pc, it1, it2)
    # the smoothed prolongator's coarse correction is the better one
    assert out[2][1] < out[3][1], (out[2][1], out[3][1])


def test_multigrid_is_bitwise_reproducible():
    t = mesh.config_large(seed=4, cells=30)
    runs = []
    for _ in range(2):
        with api.Solver(t, precond=2, deterministic=True) as s:
            s.set_growth_rates(t.rates)
            its = [s.newton_step(t.dt)["krylov_total"] for _ in range(2)]
            runs.append((s.positions(), its))
    assert np.array_equal(runs[0][0], runs[1][0]) and runs[0][1] == runs[1][1]


def test_multigrid_batch_matches_plain_runs():
    ts = [mesh.config_tiny(seed=301, n=9, n_layers=3, eta=100.0), mesh.config_small(seed=302),
          mesh.config_tiny(seed=303, n=6, n_layers=2, eta=100.0)]
    ts[1].eta[:] = 100.0
    steps = 2
    with api.Batch(ts, precond=2) as b:
        b.set_growth_rates()
        for _ in range(steps):
            assert b.step(ts[0].dt, allow_not_converged=False)["converged"].all()
        pos = [b.instance_positions(i).copy() for i in range(len(ts))]
    for i, t in enumerate(ts):
        with api.Solver(t, precond=1) as s:
            s.set_growth_rates(t.rates)
            for _ in range(steps):
                s.newton_step(t.dt)
            ref = s.positions()
        assert np.abs(pos[i] - ref).max() <= TOL_POS * np.abs(ref).max(), i


def test_multigrid_adjoint_matches_central_differences():
    t = mesh.config_tiny(seed=5, n=7, n_layers=2, eta=100.0)
    rng = np.random.default_rng(105)
    rate = 1e-4 * (1.0 + 0.5 * rng.uniform(-1, 1, t.n_elems))
    logE = np.log(t.E)
    xy = t.pos.reshape(-1, 3)
    c = xy[:, :2].mean(axis=0)
    params = np.array([c[0], c[1], 1.2 * xy[t.node_placement == 1, 2].mean(), 8.0])
    with api.Solver(t, newton_tol=1e-10, krylov_rtol=1e-12, deterministic=True, precond=2) as s:
        def loss(r, e):
            s.set_positions(t.pos)
            lv, sv = s.adjoint_forward(r, e, 3, t.dt, 2, params)
            return lv, sv
        _, sv = loss(rate, logE)
        gr, ge = s.adjoint_backward(sv)
        sv.free()
        d = rng.standard_normal(t.n_elems)
        h = 1e-4
        lp, a = loss(rate, logE + h * d)
        a.free()
        lm, b = loss(rate, logE - h * d)
        b.free()
        fd = (lp - lm) / (2 * h)
        assert abs(ge @ d - fd) <= 1e-6 * abs(fd)


def test_kept_coarse_levels_keep_the_newton_steps():
    """tf_options.multigrid_reuse_steps: coarse levels kept across time steps
    (the default, 4 steps, and 2) change the Krylov counts only -- the Newton
    counts and the positions (1e-8 relative) are those of a rebuild at every
    step (negative)."""
    t = mesh.config_large(seed=3, cells=40)
    res = []
    for keep in (-1, 0, 2):
        with api.Solver(t, precond=2, multigrid_reuse_steps=keep) as s:
            s.set_growth_rates(t.rates)
            outs = [s.newton_step(t.dt) for _ in range(7)]
            res.append(([o["iters"] for o in outs], s.positions()))
    for its, pos in res[1:]:
        assert its == res[0][0]
        assert np.abs(pos - res[0][1]).max() <= 1e-8 * np.abs(res[0][1]).max()
