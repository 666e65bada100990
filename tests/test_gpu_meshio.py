"""Meshes read from the reference's .mesh format, including prisms whose
reference (stress-free) shape differs from the initial node positions (a
pre-stressed start): GPU Newton steps against the oracle's, plain and batched."""
import numpy as np
import pytest

from oracle.oracle import Port
from tissuefolding_paperversion_gb300 import api, mesh, meshfile

pytestmark = pytest.mark.gpu
TOL_POS = 1e-8


def _prestressed(seed, eta):
    """A sheet whose prisms' reference shapes are 4 % shorter in z than the
    node positions (so the first step relaxes a stretch), written to and read
    back from the .mesh format."""
    t = mesh.config_tiny(seed=seed, n=6, n_layers=2, eta=eta)
    ref = t.pos.reshape(-1, 3)[t.conn.reshape(-1, 6)].copy()
    ref[:, :, 2] *= 0.96
    return mesh.Tissue(**{**t.__dict__, "ref_pos": ref.reshape(-1)})


@pytest.mark.parametrize("eta", [0.0, 100.0])
def test_prestressed_mesh_file_steps_match_oracle(tmp_path, eta):
    t0 = _prestressed(7, eta)
    path = str(tmp_path / "prestressed.mesh")
    meshfile.write_mesh_file(path, t0)
    t, _ = meshfile.load_tissue(path, E=1000.0, eta=eta)
    np.testing.assert_array_equal(t.ref_pos, t0.ref_pos)
    t.rates = t0.rates
    p = Port(t)
    with api.Solver(t) as s:
        s.set_growth_rates(t.rates)
        for k in range(3):
            out = s.newton_step(t.dt, allow_not_converged=False)
            ref = p.step(t.dt, t.rates)
            pos, want = s.positions(), p.positions()
            assert np.abs(pos - want).max() <= TOL_POS * np.abs(want).max(), k
            assert out["iters"] == ref["iters"], k
    # the relaxation moved the apical surface down
    z0 = t.pos.reshape(-1, 3)[t.node_placement == 1, 2]
    assert np.all(pos.reshape(-1, 3)[t.node_placement == 1, 2] < z0)


def test_prestressed_instances_in_a_batch():
    ts = [_prestressed(11, 100.0), mesh.config_tiny(seed=12, n=5, n_layers=2, eta=100.0)]
    with api.Batch(ts, deterministic=True) as b:
        b.set_growth_rates()
        for _ in range(2):
            b.step(ts[0].dt)
        pos = [b.instance_positions(i).copy() for i in range(2)]
    for i, t in enumerate(ts):
        with api.Solver(t, deterministic=True) as s:
            s.set_growth_rates(t.rates)
            for _ in range(2):
                s.newton_step(t.dt)
            assert np.array_equal(pos[i], s.positions()), i


def test_frames_written_during_a_run(tmp_path):
    t = mesh.config_tiny(seed=13, n=4, n_layers=2)
    path = str(tmp_path / "Save_Frame")
    with api.Solver(t) as s:
        s.set_growth_rates(t.rates)
        for k in range(3):
            s.newton_step(t.dt)
            api.write_frame(path, (k + 1) * t.dt, s.positions(), t.conn, t.node_placement, append=k > 0)
        last = s.positions()
    lines = open(path).read().splitlines()
    per = 4 + t.n_nodes + t.n_elems
    assert len(lines) == 3 * per
    blk = lines[2 * per:3 * per]
    xyz = np.array([[float(ln[20 * d:20 * (d + 1)]) for d in range(3)] for ln in blk[2:2 + t.n_nodes]])
    np.testing.assert_allclose(xyz.reshape(-1), last, rtol=1e-9, atol=1e-12)
