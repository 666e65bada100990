"""The packing restatement (oracle/packing.py) against fixtures generated by
the reference's own node, prism and solver classes (tests/golden/
make_golden.py --only-packing) and, where the reference checkout is present,
against the reference driver directly.  CPU only."""
import os

import numpy as np
import pytest

from oracle import packing as op
from tissuefolding_paperversion_gb300 import mesh

GOLD = os.path.join(os.path.dirname(__file__), "golden")
CASES = [("steps_facing_packing", dict(seed=12, gap=1.5, E=100000.0, eta=0.0)),
         ("steps_facing_packing_viscous", dict(seed=13, gap=1.5, E=100000.0, eta=100.0))]


def _masses(t):
    vref = op.reference_volumes(t.pos.reshape(-1, 3)[t.conn.reshape(-1, 6)])
    return op.node_masses(t.conn, t.n_nodes, vref, np.tile(np.eye(3), (t.n_elems, 1, 1)))


@pytest.mark.parametrize("name,kw", CASES)
def test_detection_and_forces_match_the_reference_fixture(name, kw):
    f = np.load(os.path.join(GOLD, name + ".npz"))
    t = mesh.config_facing_sheets(**kw)
    uk, un = mesh.perturbed_state(t, seed=7, amp=0.05)
    m = _masses(t)
    np.testing.assert_array_equal(m, f["asm_masses"])
    pk = op.detect(un, t.conn, t.node_placement, m, bool(f["drop_last_segment"]))
    np.testing.assert_array_equal(pk["nodes"], f["asm_nodes"])
    np.testing.assert_array_equal(pk["w"], f["asm_w"])
    np.testing.assert_array_equal(pk["mbar"], f["asm_mbar"])
    assert pk["threshold"] == float(f["asm_threshold"])
    force, trip = op.forces_and_jacobian(uk, pk)
    np.testing.assert_allclose(force, f["asm_forces"], rtol=0, atol=1e-13 * np.abs(f["asm_forces"]).max())
    assert len(trip) == 12 * len(pk["nodes"])


def test_reference_merge_leaves_out_the_last_segment():
    t = mesh.config_facing_sheets(seed=12, gap=1.5, E=100000.0)
    m = _masses(t)
    kept = op.detect(t.pos, t.conn, t.node_placement, m, drop_last_segment=False)
    merged = op.detect(t.pos, t.conn, t.node_placement, m, drop_last_segment=True)
    last = (t.n_nodes // (t.n_nodes // 16) - 1) * (t.n_nodes // 16)
    lost = kept["nodes"][kept["nodes"][:, 0] >= last]
    assert len(lost) > 0 and len(merged["nodes"]) == len(kept["nodes"]) - len(lost)
    assert not np.any(merged["nodes"][:, 0] >= last)


def test_couples_are_same_surface_non_neighbours_within_the_distance():
    t = mesh.config_facing_sheets(seed=3, n=12, gap=1.5, E=100000.0)
    pk = op.detect(t.pos, t.conn, t.node_placement, _masses(t), drop_last_segment=False)
    p = t.pos.reshape(-1, 3)
    a, b = pk["nodes"][:, 0], pk["nodes"][:, 1]
    assert len(a) > 0 and np.all(a < b)
    assert np.all(t.node_placement[a] == t.node_placement[b])
    d = np.linalg.norm(p[a] - p[b], axis=1)
    assert np.all(d < pk["detect"])
    np.testing.assert_allclose(np.linalg.norm(pk["w"], axis=1), 1.0, rtol=1e-14)
    nb = op.neighbours(t.conn, t.n_nodes)
    assert not any(int(j) in nb[int(i)] for i, j in zip(a, b))


def test_jacobian_is_minus_the_force_derivative():
    t = mesh.config_facing_sheets(seed=5, gap=1.5, E=100000.0)
    pk = op.detect(t.pos, t.conn, t.node_placement, _masses(t))
    uk, _ = mesh.perturbed_state(t, seed=9, amp=0.05)
    n3 = 3 * t.n_nodes
    K = np.zeros((n3, n3))
    for r, c, v in op.forces_and_jacobian(uk, pk)[1]:
        K[r, c] += v
    rng = np.random.default_rng(1)
    d = rng.standard_normal(n3)
    h = 1e-6
    fp = op.forces_and_jacobian(uk + h * d, pk)[0]
    fm = op.forces_and_jacobian(uk - h * d, pk)[0]
    np.testing.assert_allclose(K @ d, -(fp - fm) / (2 * h), rtol=1e-6, atol=1e-6 * np.abs(K @ d).max())


def test_restatement_matches_the_reference_driver_when_present():
    from oracle.oracle import Ref

    if not Ref.available():
        pytest.skip("reference checkout not present")
    for seed in (2, 12):
        t = mesh.config_facing_sheets(seed=seed, gap=1.5, E=100000.0)
        r = Ref(t)
        try:
            for drop in (True, False):
                r.set_packing(True, drop)
                r.pack_detect()
                got = r.packing()
                want = op.detect(t.pos, t.conn, t.node_placement, _masses(t), drop)
                np.testing.assert_array_equal(got["nodes"], want["nodes"])
                np.testing.assert_array_equal(got["w"], want["w"])
                assert got["threshold"] == want["threshold"]
                np.testing.assert_array_equal(r.node_masses(), _masses(t))
        finally:
            r.close()


def _node0_at_max_x(t):
    """The same sheets renumbered so that node 0 alone holds the largest x."""
    t = mesh.swap_nodes(t, 0, int(np.argmax(t.pos.reshape(-1, 3)[:, 0])))
    t.pos[0] += 0.3
    return t


def test_reference_box_when_node_0_holds_the_maximum():
    """The reference's bounding box never tests node 0 for the maximum; the
    restatement keeps that, and it changes which first nodes find couples."""
    from oracle.oracle import Ref
    from oracle.growth import bounding_box

    t = _node0_at_max_x(mesh.config_facing_sheets(seed=8, n=9, gap=1.5, E=100000.0, offset=(0.4, 0.2)))
    p = t.pos.reshape(-1, 3)
    lo, size = bounding_box(p)
    assert lo[0] + size[0] < p[:, 0].max()
    want = op.detect(t.pos, t.conn, t.node_placement, _masses(t), True)
    assert len(want["nodes"]) > 0 and 0 not in want["nodes"][:, 0]
    if not Ref.available():
        pytest.skip("reference checkout not present")
    r = Ref(t)
    try:
        r.set_packing(True, True)
        r.pack_detect()
        got = r.packing()
        np.testing.assert_array_equal(got["nodes"], want["nodes"])
        np.testing.assert_array_equal(got["w"], want["w"])
    finally:
        r.close()
