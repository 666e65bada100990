"""The checked build (libtfgpu_checked.so, -DTF_CHECKED): every checked index
of the main kernels -- prism node ids and scatter offsets, Krylov and
smoother columns, extra-block columns, multigrid transfers, packing couples,
growth-update gathers --
is tested before its access and a failure is reported as TF_CUDA_ERROR
instead of touching memory out of bounds.  The same workloads through the
checked and the normal library must flag nothing and agree bit for bit
(deterministic assembly; the tests add no arithmetic), the adjoint up to the
order of its atomic carry additions."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKLOADS = r'''
import json, sys
import numpy as np
sys.path.insert(0, ROOT)
from tissuefolding_paperversion_gb300 import api, mesh
out = {}
t = mesh.config_small(seed=0)
for pc in (1, 2):
    with api.Solver(t, precond=pc, deterministic=True) as s:
        s.set_growth_rates(t.rates)
        its = [s.newton_step(t.dt, allow_not_converged=False)["krylov_total"] for _ in range(2)]
        out[f"small{pc}"] = [s.positions().tolist(), its]
t = mesh.config_facing_sheets(seed=12, gap=1.5, E=100000.0)
with api.Solver(t, precond=2, deterministic=True) as s:
    s.set_growth_rates(t.rates)
    s.set_packing(True)
    its = [s.newton_step(t.dt)["krylov_total"] for _ in range(2)]
    out["packing"] = [s.positions().tolist(), its]
from oracle import growth as og
t, start, fns = og.rotated_case()
with api.Solver(t, deterministic=True) as s:
    og.add_functions(s, fns + og.mixed_case()[1][1:2])
    s.set_growth_rates(t.rates)
    s.set_positions(start)
    its = [s.newton_step(t.dt)["krylov_total"] for _ in range(2)]
    out["growth"] = [s.positions().tolist(), s.get_Fg()[0].tolist(), its]
ts = [mesh.config_tiny(seed=301, n=9, n_layers=3, eta=100.0), mesh.config_tiny(seed=303, n=6, n_layers=2)]
with api.Batch(ts, precond=2, deterministic=True) as b:
    b.set_growth_rates()
    b.step(ts[0].dt)
    out["batch"] = [b.instance_positions(i).tolist() for i in range(2)]
t = mesh.config_tiny(seed=5, n=5, n_layers=2, eta=100.0)
with api.Solver(t, deterministic=True, krylov_rtol=1e-12) as s:
    xy = t.pos.reshape(-1, 3)
    params = np.array([xy[:, 0].mean(), xy[:, 1].mean(), 12.0, 8.0])
    lv, sv = s.adjoint_forward(np.full(t.n_elems, 1e-5), np.log(t.E), 3, t.dt, 2, params)
    gr, ge = s.adjoint_backward(sv)
    sv.free()
    out["adjoint"] = [lv, gr.tolist(), ge.tolist()]
print(json.dumps(out))
'''


def _run(checked):
    env = dict(os.environ)
    env["TF_CHECKED"] = "1" if checked else "0"
    code = "ROOT = " + repr(ROOT) + "\n" + WORKLOADS
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_checked_build_flags_nothing_and_matches_the_normal_build():
    from tissuefolding_paperversion_gb300 import build

    build.build(checked=True)
    got = _run(True)
    want = _run(False)
    assert got.keys() == want.keys()
    for k in want:
        if k == "adjoint":
            # the adjoint's carry to the previous step is scattered with atomics:
            # equal up to the order of its additions
            assert got[k][0] == want[k][0]
            for a, b in zip(got[k][1:], want[k][1:]):
                np.testing.assert_allclose(a, b, rtol=1e-11, atol=1e-11 * np.abs(b).max())
        else:
            assert got[k] == want[k], k
