"""Workload generator: sizes, orientation and boundary data of the configs."""
import numpy as np

from tissuefolding_paperversion_gb300 import mesh


def _orientation_ok(t):
    p = t.pos.reshape(-1, 3)
    c = t.conn.reshape(-1, 6)
    v1 = p[c[:, 1]] - p[c[:, 0]]
    v2 = p[c[:, 2]] - p[c[:, 0]]
    view = p[c[:, 0]] - p[c[:, 3]]
    # Prism::checkRotationConsistency3D (Prism.cpp:364-412) swaps when > 0
    return (np.einsum("ij,ij->i", view, np.cross(v1, v2)) < 0).all()


def test_small_sizes():
    t = mesh.config_small()
    assert t.n_nodes == 1323 and t.n_elems == 1600
    assert 3 * t.n_nodes == 3969
    assert _orientation_ok(t)
    pl = t.node_placement
    assert (pl == 0).sum() == 441 and (pl == 1).sum() == 441
    assert t.fixed.reshape(-1, 3)[pl == 0, 2].all() and not t.fixed.reshape(-1, 3)[:, :2].any()
    r = t.rates.reshape(-1, 3)
    assert np.allclose(np.unique(np.round(r[:, 0] * 3600, 6)), [0.01, 0.015])


def test_large_sizes():
    t = mesh.config_large()
    assert t.n_nodes == 202005 and t.n_elems == 320000
    assert _orientation_ok(t)
    assert (t.eta == 100.0).all()
    assert abs(np.log(t.E).std() - 0.3) < 0.01


def test_batch_instance_range():
    for s in range(4):
        t = mesh.config_batch_instance(s)
        assert 500 <= t.n_elems <= 60000
        assert _orientation_ok(t)


def test_seeded_reproducible():
    a, b = mesh.config_small(seed=3), mesh.config_small(seed=3)
    assert (a.pos == b.pos).all() and (a.conn == b.conn).all()
