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
