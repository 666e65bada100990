"""Failure paths of the C ABI on the GPU: every one returns a status code and
leaves the context usable.  Failures are made on the host (bad inputs, tiny
iteration caps, a singular system, a non-finite position); nothing here
faults or traps the GPU."""
import numpy as np
import pytest

from tissuefolding_paperversion_gb300 import api, mesh

pytestmark = pytest.mark.gpu


def test_newton_cap_returns_not_converged_and_advances():
    t = mesh.config_tiny(seed=101, n=4, n_layers=2)
    t.rates = t.rates * 50.0
    # max_iter = 1 allows two solves (Simulation.cpp:6568: stop when k > max)
    with api.Solver(t, newton_max_iter=1) as s:
        s.set_growth_rates(t.rates)
        out = s.newton_step(t.dt, allow_not_converged=True)
        assert out["status"] == api.TF_NOT_CONVERGED
        assert out["iters"] == 2 and not out["converged"]
        assert not np.array_equal(s.positions(), t.pos)
        out2 = s.newton_step(t.dt, allow_not_converged=True)   # context still usable
        assert out2["status"] in (api.TF_OK, api.TF_NOT_CONVERGED)


def test_krylov_cap_returns_status():
    t = mesh.config_small(seed=4)
    uk, un = mesh.perturbed_state(t, seed=5)
    with api.Solver(t, krylov_max_iter=2) as s:
        s.set_state(uk, un, t.dt)
        s.assemble()
        out = s.solve(allow_not_converged=True)
        assert out["status"] == api.TF_KRYLOV_NOT_CONVERGED and out["iters"] == 2


def test_non_finite_position_is_reported():
    t = mesh.config_tiny(seed=102, n=4, n_layers=2)
    uk, un = mesh.perturbed_state(t, seed=6)
    uk[7] = np.nan
    with api.Solver(t) as s:
        s.set_state(uk, un, t.dt)
        s.assemble()
        with pytest.raises(api.TfError) as e:
            s.solve()
        assert e.value.status == api.TF_NAN_DETECTED
        s.set_state(un, un, t.dt)          # recovers
        s.assemble()
        assert s.solve()["status"] == api.TF_OK


def test_singular_system_does_not_hang():
    # no fixed DOF and no external viscosity: rigid motions make K singular
    t = mesh.config_tiny(seed=103, n=4, n_layers=2)
    t.fixed[:] = 0
    t.ext_visc[:] = 0.0
    uk, un = mesh.perturbed_state(t, seed=7)
    with api.Solver(t, krylov_max_iter=500) as s:
        s.set_state(uk, un, t.dt)
        s.assemble()
        try:
            out = s.solve(allow_not_converged=True)
            assert out["status"] in (api.TF_OK, api.TF_KRYLOV_NOT_CONVERGED)
        except api.TfError as e:  # a breakdown is reported, not hung on
            assert e.status == api.TF_KRYLOV_BREAKDOWN
        s.set_state(un, un, t.dt)
        s.assemble()
