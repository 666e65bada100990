"""The Newton loop on the device: after the first Newton iteration of a step
(host-driven: the multigrid rebuild, the element-tile autotuning, any
retries), the remaining iterations run as one graph launch -- a conditional
while node over assembly, the Krylov solve (itself a nested while node), the
Newton test of every instance and the update (tf_step_stats.device_iters).
Configurations that keep host work between iterations (packing, bound DOFs)
stay host-driven.  Results are checked against the reference elsewhere
(tests/test_gpu_parity.py, tests/test_gpu_large_parity.py run through this
loop); here: that the loop runs, that a batch run through it (the instance
masks updated on the device) reproduces each instance's plain run, and that
packing keeps the host loop."""
import numpy as np
import pytest

from tissuefolding_paperversion_gb300 import api, mesh

pytestmark = pytest.mark.gpu


def test_device_loop_runs_the_iterations_after_the_first():
    t = mesh.config_small(seed=0)
    with api.Solver(t) as s:
        s.set_growth_rates(t.rates)
        for k in range(3):
            out = s.newton_step(t.dt, allow_not_converged=False)
            assert out["iters"] >= 2
            assert out["device_iters"] == out["iters"] - 1, (k, out)


def test_device_loop_in_a_batch_masks_instances():
    ts = [mesh.config_tiny(seed=301, n=4, n_layers=2), mesh.config_small(seed=302),
          mesh.config_tiny(seed=303, n=6, n_layers=3)]
    ts[2].rates = ts[2].rates * 8.0  # more Newton iterations than the others
    with api.Batch(ts) as b:
        b.set_growth_rates()
        counts = []
        for _ in range(2):
            out = b.step(ts[0].dt, allow_not_converged=False)
            assert out["device_iters"] == int(np.max(out["iters"])) - 1, out
            counts.append(out["iters"].copy())
        pos = [b.instance_positions(i).copy() for i in range(len(ts))]
    assert counts[0][2] > counts[0][0]  # the masks kept instances apart
    # each instance as a plain run: same Newton counts, same positions (1e-12)
    for i, t in enumerate(ts):
        with api.Solver(t) as s:
            s.set_growth_rates(t.rates)
            its = [s.newton_step(t.dt)["iters"] for _ in range(2)]
            p = s.positions()
        assert its == [c[i] for c in counts], i
        assert np.abs(p - pos[i]).max() <= 1e-12 * np.abs(p).max(), i


def test_packing_keeps_the_host_loop():
    t = mesh.config_facing_sheets(seed=12, gap=1.5, E=1e5, eta=0.0)
    with api.Solver(t) as s:
        s.set_growth_rates(t.rates)
        s.set_packing(True)
        out = s.newton_step(t.dt)
        assert out["device_iters"] == 0
        assert out["iters"] >= 2


def test_host_loops_option_gives_the_same_steps():
    """tf_options.host_loops (host-checked Krylov chunks, host-driven Newton
    iterations: what a profiler that cannot see inside conditional graph nodes
    needs) takes the same Newton steps."""
    t = mesh.config_large(seed=0, cells=40)
    res = []
    for host in (False, True):
        with api.Solver(t, precond=2, host_loops=host) as s:
            s.set_growth_rates(t.rates)
            outs = [s.newton_step(t.dt) for _ in range(2)]
            res.append(([o["iters"] for o in outs], s.positions(), [o["device_iters"] for o in outs]))
    assert res[0][0] == res[1][0]
    assert res[1][2] == [0, 0] and all(d > 0 for d in res[0][2])
    assert np.abs(res[0][1] - res[1][1]).max() <= 1e-12 * np.abs(res[1][1]).max()
