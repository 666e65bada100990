"""Bound DOFs (slave/master couples): Newton steps against the reference's own
NewtonRaphsonSolver run with the same couples (golden fixture generated by
tests/golden/make_golden.py from the reference's sources)."""
import os

import numpy as np
import pytest

from tissuefolding_paperversion_gb300 import api, mesh

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("precond", [1, 2])
def test_bound_steps_match_reference(precond):
    f = np.load(os.path.join(GOLD, "steps_tiny_bound.npz"))
    t = mesh.config_tiny(seed=15, n=5, n_layers=2, eta=100.0)
    with api.Solver(t, precond=precond, krylov_rtol=1e-12) as s:
        s.set_growth_rates(t.rates)
        s.set_dof_bindings(f["slaves"], f["masters"])
        for k in range(f["positions"].shape[0]):
            out = s.newton_step(t.dt, allow_not_converged=False)
            ref = f["positions"][k]
            pos = s.positions()
            assert np.abs(pos - ref).max() <= 1e-8 * np.abs(ref).max(), (k, np.abs(pos - ref).max())
            assert out["iters"] == f["iters"][k], (k, out["iters"])
    # the couples moved together: equal displacements of slave and master
    d = pos - t.pos
    np.testing.assert_allclose(d[f["slaves"]], d[f["masters"]], rtol=0, atol=1e-12)


def test_bindings_are_validated():
    t = mesh.config_tiny(seed=16, n=4, n_layers=2)
    with api.Solver(t) as s:
        with pytest.raises(api.TfError):
            s.set_dof_bindings([3 * t.n_nodes], [0])
        with pytest.raises(api.TfError):
            s.set_dof_bindings([5], [5])
        s.set_dof_bindings([], [])


def _csr_dense(ia, ja, a, n):
    K = np.zeros((n, n))
    for r in range(n):
        K[r, ja[ia[r]:ia[r + 1]]] = a[ia[r]:ia[r + 1]]
    return K


def test_device_merges_equal_the_reference_rule():
    """The merges run on the device (a plan built once per couple list and
    extra-block layout) and give N^T K N + I and N^T g exactly as
    NewtonRaphsonSolver::calculateBoundKWithSlavesMasterDoF
    (NewtonRaphsonSolver.cpp:154-235) forms them on the dense K; a second
    assembly and solve reuse the plan."""
    f = np.load(os.path.join(GOLD, "steps_tiny_bound.npz"))
    t = mesh.config_tiny(seed=15, n=5, n_layers=2, eta=100.0)
    uk, un = mesh.perturbed_state(t, seed=17, amp=0.1)
    n = 3 * t.n_nodes
    with api.Solver(t, precond=1, krylov_rtol=1e-12) as s:
        s.set_dof_bindings(f["slaves"], f["masters"])
        for _ in range(2):
            s.set_state(uk, un, t.dt)
            s.assemble()
            K = _csr_dense(*s.export_csr(0.0), n)
            g = s.residual()
            s.solve()
            Kb = _csr_dense(*s.export_csr(0.0), n)
            gb = s.residual()
            du = s.delta_u()
    for sd, md in zip(f["slaves"], f["masters"]):
        g[md] += g[sd]
        g[sd] = 0.0
        K[md, :] += K[sd, :]
        K[sd, :] = 0.0
        K[:, md] += K[:, sd]
        K[:, sd] = 0.0
        K[sd, sd] = 1.0
    assert np.abs(Kb - K).max() <= 1e-14 * np.abs(K).max()
    assert np.abs(gb - g).max() <= 1e-14 * np.abs(g).max()
    # the bound system is solved (A = K^T; a slave's row and column of the bound
    # matrix are the unit vector and its g is zero, so its solved update is
    # zero), and then the slaves follow their masters
    du0 = du.copy()
    du0[f["slaves"]] = 0.0
    assert np.abs(K.T @ du0 - g).max() <= 1e-9 * np.abs(g).max()
    np.testing.assert_array_equal(du[f["slaves"]], du[f["masters"]])
