"""Batches: many tissues in one handle, one launch sequence, per-instance
Krylov scalars, convergence masks and Newton counts.  Each batched instance
must reproduce its own plain run: bit for bit with the order-fixed assembly
(same element order, same per-instance reduction order), and to 1e-12 with
the atomic scatter."""
import numpy as np
import pytest

from tissuefolding_paperversion_gb300 import api, mesh

pytestmark = pytest.mark.gpu


def _instances(eta=0.0):
    ts = [mesh.config_tiny(seed=201, n=4, n_layers=2, eta=eta),
          mesh.config_tiny(seed=202, n=7, n_layers=3, eta=eta),
          mesh.config_small(seed=203),
          mesh.config_tiny(seed=204, n=5, n_layers=2, eta=eta)]
    ts[2].eta[:] = eta
    ts[3].rates = ts[3].rates * 8.0      # needs more Newton iterations
    return ts


def _plain(t, steps, deterministic):
    with api.Solver(t, deterministic=deterministic) as s:
        s.set_growth_rates(t.rates)
        its = [s.newton_step(t.dt)["iters"] for _ in range(steps)]
        return s.positions(), its


@pytest.mark.parametrize("deterministic", [True, False])
def test_batch_reproduces_plain_runs(deterministic):
    ts = _instances()
    steps = 3
    with api.Batch(ts, deterministic=deterministic) as b:
        b.set_growth_rates()
        counts = [b.step(ts[0].dt)["iters"].copy() for _ in range(steps)]
        pos = [b.instance_positions(i).copy() for i in range(len(ts))]
    for i, t in enumerate(ts):
        ref, its = _plain(t, steps, deterministic)
        assert [c[i] for c in counts] == its, i
        if deterministic:
            assert np.array_equal(pos[i], ref), i
        else:
            assert np.abs(pos[i] - ref).max() <= 1e-12 * np.abs(ref).max(), i
    # the fast-growing instance iterated more than the others in at least one step
    assert max(c[3] for c in counts) > min(c[0] for c in counts)


def test_batch_with_viscous_instances():
    ts = _instances(eta=100.0)
    with api.Batch(ts) as b:
        b.set_growth_rates()
        for _ in range(2):
            out = b.step(ts[0].dt, allow_not_converged=False)
            assert out["converged"].all()
        pos = [b.instance_positions(i).copy() for i in range(len(ts))]
    for i, t in enumerate(ts):
        ref, _ = _plain(t, 2, False)
        assert np.abs(pos[i] - ref).max() <= 1e-8 * np.abs(ref).max(), i


def test_autotuner_picks_a_valid_tile():
    with api.Batch(_instances()) as b:
        b.set_growth_rates()
        b.step(60.0)
        assert b.elements_per_cta() in (8, 16, 32)


def test_solve_autotuner_picks_valid_variants():
    """The solve's kernel variants are timed on the handle's own matrix before
    its first solve (FP64 SpMV: 1, 2 or 4 slots in flight per lane; level-0
    smoother: 2, 4 or 8) and the solution does not depend on the choice."""
    t = mesh.config_large(seed=0, cells=40)
    res = []
    for autotune in (True, False):
        with api.Solver(t, precond=2, autotune=autotune) as s:
            s.set_growth_rates(t.rates)
            its = [s.newton_step(t.dt)["iters"] for _ in range(2)]
            v = s.tiles()
            res.append((its, s.positions()))
        if autotune:
            assert v["spmv_unroll"] in (1, 2, 4) and v["smoother_unroll"] in (2, 4, 8), v
        else:
            assert v["spmv_unroll"] == 2 and v["smoother_unroll"] == 4, v
    assert res[0][0] == res[1][0]
    assert np.abs(res[0][1] - res[1][1]).max() <= 1e-12 * np.abs(res[1][1]).max()
