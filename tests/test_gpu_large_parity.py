"""Twenty implicit steps of the 320,000-prism sheet on the GPU against the
oracle's run of the same steps (tests/golden/steps_large_320k.npz, made by
tests/golden/make_large_steps.py: the oracle's restatement of the reference's
element loop, scatter order, boundary conditions and Newton loop, with
sparse storage and the Pardiso stand-in solve, because the reference's
dense K would take 2.94 TB at this size).

Per step: the Newton iteration count must be identical, ||du|| of every
iteration must agree to 1e-6 of the step's first update (a later update
corrects the error the earlier linear solves left, so its own norm carries
that error: the GPU's Krylov solves stop at a relative residual of 1e-8,
the oracle's at a backward error of 1e-14), and the positions of 2,048
seeded nodes must lie
within 1e-8 of the oracle's relative to the largest coordinate, with the
block-Jacobi preconditioner and with the smoothed-aggregation multigrid
(FP32 V-cycle, FP16 level-0 smoother operator)."""
import os

import numpy as np
import pytest

from tissuefolding_paperversion_gb300 import api, mesh

pytestmark = pytest.mark.gpu
FIXTURE = os.path.join(os.path.dirname(__file__), "golden", "steps_large_320k.npz")
TOL_POS = 1e-8      # positions after every step, relative to the largest coordinate
TOL_DU = 1e-6       # ||du|| of every Newton iteration, relative to the step's first update


@pytest.mark.skipif(not os.path.exists(FIXTURE), reason="the 320k-prism oracle run is not committed")
@pytest.mark.parametrize("precond", [1, 2], ids=["block-jacobi", "multigrid"])
def test_twenty_steps_of_the_320k_sheet_match_the_oracle(precond):
    f = np.load(FIXTURE)
    t = mesh.config_large(seed=int(f["seed"]), cells=int(f["cells"]))
    assert t.n_elems == int(f["n_prisms"]) and t.n_nodes == int(f["n_nodes"])
    sample = f["sample_nodes"]
    scale = np.abs(f["sample_positions"]).max()
    pos0 = t.pos.reshape(-1, 3)
    worst = 0.0
    with api.Solver(t, precond=precond) as s:
        s.set_growth_rates(t.rates)
        for k in range(f["iters"].shape[0]):
            out = s.newton_step(t.dt, allow_not_converged=False)
            p = s.positions().reshape(-1, 3)
            assert out["iters"] == f["iters"][k], (k, out["iters"], f["iters"][k])
            ref_du = f["dunorm"][k][: f["iters"][k]]
            got_du = np.asarray(out["dunorm"])[: out["iters"]]
            assert np.all(np.abs(got_du - ref_du) <= TOL_DU * ref_du[0]), (k, got_du, ref_du)
            assert got_du[-1] <= 1e-8 and ref_du[-1] <= 1e-8
            err = np.abs(p[sample] - f["sample_positions"][k]).max() / scale
            worst = max(worst, err)
            assert err <= TOL_POS, (k, err)
            # whole-sheet checks: the mean position and the displacement norm
            assert np.abs(p.mean(axis=0) - f["position_sums"][k] / t.n_nodes).max() <= TOL_POS * scale, k
            dn = np.linalg.norm(p - pos0)
            assert abs(dn - f["disp_norm"][k]) <= 1e-7 * f["disp_norm"][k], (k, dn, f["disp_norm"][k])
    print(f"precond {precond}: worst relative position error over 20 steps {worst:.2e}")
