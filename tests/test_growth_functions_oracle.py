"""The growth-function oracle (oracle/growth.py) pinned against the
reference: the committed fixtures (made by the reference's own
UniformGrowthFunction, RingGrowthFunction, GridBasedGrowthFunction and
ShapeBase::calculateFgFromRates / calculateFgFromGridCorners) and, where the
reference builds here, the reference driver directly."""
from __future__ import annotations

import math
import os

import numpy as np
import pytest

from oracle import growth as G
from oracle.oracle import Ref
from tissuefolding_paperversion_gb300 import mesh

GOLD = os.path.join(os.path.dirname(__file__), "golden")
NAMES = G.FIXTURES
grid_case = G.fixture_case


def oracle_for(t, fns, interp, pinned):
    o = G.GridGrowthOracle(t.pos, t.conn, t.node_placement)
    for f in fns:
        o.add(**f)
    o.interp, o.pinned = interp, pinned
    return o


@pytest.mark.parametrize("name", NAMES)
def test_fixture_inputs_are_rebuilt(name):
    f = np.load(os.path.join(GOLD, name + ".npz"))
    t, fns, interp, pinned = grid_case(name)
    assert int(f["n_fns"]) == len(fns) and int(f["interp"]) == interp and bool(f["pinned"]) == pinned
    for i, fn in enumerate(fns):
        np.testing.assert_array_equal(f[f"fn{i}_rates"], fn["rates"])
        np.testing.assert_array_equal(f[f"fn{i}_angles"], fn["angles_deg"])


@pytest.mark.parametrize("name", NAMES)
def test_positions_match_the_reference_bit_for_bit(name):
    f = np.load(os.path.join(GOLD, name + ".npz"))
    t, fns, interp, pinned = grid_case(name)
    o = oracle_for(t, fns, interp, pinned)
    np.testing.assert_array_equal(o.state["relz"], f["relz"])
    np.testing.assert_array_equal(o.state["rel0"], f["rel0"])
    cur = G.relative_positions(t.pos, t.conn, o.state["src"])
    np.testing.assert_array_equal(cur, f["rel"])


@pytest.mark.parametrize("name", NAMES)
def test_one_growth_update_matches_the_reference(name):
    f = np.load(os.path.join(GOLD, name + ".npz"))
    t, fns, interp, pinned = grid_case(name)
    o = oracle_for(t, fns, interp, pinned)
    Fg = o.grow(np.broadcast_to(np.eye(3), (t.n_elems, 3, 3)), t.pos, 0.0, t.dt, t.rates)
    assert np.abs(Fg.reshape(-1) - f["Fg_grow"]).max() <= 1e-15
    assert np.abs(f["Fg_grow"] - np.tile(np.eye(3).reshape(-1), t.n_elems)).max() > 1e-3  # it does grow


def test_reference_box_misses_the_maximum_held_by_node_0():
    t, _, _, _ = grid_case("steps_grid_growth")
    p = t.pos.reshape(-1, 3)
    assert p[0, 0] > p[1:, 0].max()
    lo, size = G.bounding_box(t.pos)
    assert lo[0] == p[:, 0].min()
    assert lo[0] + size[0] < p[0, 0]        # node 0 never tested for the maximum
    cx = G.centres(t.pos, t.conn)[:, 0]
    quirk = G.relative_positions(t.pos, t.conn, np.arange(t.n_elems))[:, 0]
    true_box = (cx - p[:, 0].min()) / (p[:, 0].max() - p[:, 0].min())
    assert np.abs(quirk - true_box).max() > 1e-3


def test_column_rule_takes_the_apical_position():
    t, _, _, _ = grid_case("steps_grid_growth")
    o = G.GridGrowthOracle(t.pos, t.conn, t.node_placement)
    assert o.state["layers"] == 4
    place = G.element_placement(t.conn, t.node_placement)
    src = o.state["src"]
    moved = np.nonzero(src != np.arange(t.n_elems))[0]
    assert moved.size == 2 * (place == 1).sum()          # layers 0 and 1 of each column
    assert (place[src[moved]] == 1).all()
    assert math.isclose(o.state["height"], 20.0, rel_tol=1e-12)


def test_compatible_corners_flip_and_eliminate():
    r = np.array([[[2.0, 1.0, 0.0], [1.0, 1.05, 0.0]],
                  [[2.0, 1.0, 0.0], [3.0, 1.0, 0.5]]])      # [i][j]: (0,0) (0,1) / (1,0) (1,1)
    a = np.array([[10.0, 50.0], [100.0, 190.0]])
    cg, ca, ce = G.compatible_corners(r, a)
    # corner order (0,0), (1,0), (0,1), (1,1)
    np.testing.assert_array_equal(ce[0, 0], [False, False, True, False])
    d = math.pi / 180.0
    assert math.isclose(ca[0, 0, 0], 10 * d) and math.isclose(ca[0, 0, 1], 10 * d)   # 100 deg turned by -90
    np.testing.assert_array_equal(cg[0, 0, 1], [1.0, 2.0, 0.0])                     # ... so x and y swap
    assert ca[0, 0, 2] == 0.0                                                        # no angle
    assert math.isclose(ca[0, 0, 3], 10 * d, abs_tol=1e-15)                          # 190 -> 10 deg
    np.testing.assert_array_equal(cg[0, 0, 3], [3.0, 1.0, 0.5])


def test_grid_index_clamps_like_the_reference():
    rel = np.array([[0.0, 0.0], [1.0, 1.0], [-0.1, 0.5], [0.999999, 1.2], [0.5, 0.25]])
    ix, iy, fx, fy = G.grid_index(rel, 5, 3)
    np.testing.assert_array_equal(ix, [0, 3, 0, 3, 2])
    np.testing.assert_array_equal(fx[[1, 2]], [1.0, 0.0])
    np.testing.assert_array_equal(iy, [0, 1, 1, 1, 0])
    assert fy[3] == 1.0 and fy[4] == 0.5


ref_only = pytest.mark.skipif(not Ref.available(), reason="the reference driver is not built here")


@ref_only
@pytest.mark.parametrize("interp,pinned,window", [(0, False, (-1e30, 1e30)), (1, False, (-1e30, 1e30)),
                                                  (0, True, (-1e30, 1e30)), (1, True, (0.0, 30.0))])
def test_oracle_matches_the_reference_driver(interp, pinned, window):
    t = mesh.config_tiny(seed=3, n=6, n_layers=4, jitter=0.6)
    rng = np.random.default_rng(interp + 2 * pinned)
    rates, ang = mesh.grid_growth_inputs(40 + interp, 5, 4)
    R = Ref(t)
    R.add_grid_growth(rates, ang, window[0], window[1], 0.2, 0.8)
    R.set_grid_mode(interp, pinned)
    o = G.GridGrowthOracle(t.pos, t.conn, t.node_placement)
    o.add(rates, ang, window[0], window[1], 0.2, 0.8)
    o.interp, o.pinned = interp, pinned
    rr = rng.uniform(0, 1e-5, size=3 * t.n_elems)
    for time in (0.0, 45.0):
        R.time = time
        F0 = R.get_Fg()[0]
        R.grow(60.0, rr)
        F1 = R.get_Fg()[0]
        Fo = o.grow(F0.reshape(-1, 3, 3), t.pos, time, 60.0, rr)
        assert np.abs(F1.reshape(-1, 3, 3) - Fo).max() <= 1e-15
    R.close()


@ref_only
def test_repin_matches_the_reference_driver():
    t = mesh.config_tiny(seed=4, n=5, n_layers=3)
    rates, ang = mesh.grid_growth_inputs(50, 4, 4)
    R = Ref(t)
    R.add_grid_growth(rates, ang)
    moved = t.pos + np.random.default_rng(1).uniform(-0.5, 0.5, size=t.pos.shape)
    R.set_positions(moved)
    R.repin_grid_growth()
    _, rel0, _ = R.grid_positions()
    o = G.GridGrowthOracle(t.pos, t.conn, t.node_placement)
    o.repin(moved)
    np.testing.assert_array_equal(rel0, o.state["rel0"])
    R.close()


def test_mixed_functions_match_the_reference():
    f = np.load(os.path.join(GOLD, G.MIXED_FIXTURE + ".npz"))
    t, fns = G.mixed_case()
    o = G.GrowthOracle(t.pos, t.conn, t.node_placement)
    G.add_functions(o, fns)
    Fg = o.grow(np.eye(3), t.pos, 0.0, t.dt, t.rates)
    assert np.abs(Fg.reshape(-1) - f["Fg_grow"]).max() <= 1e-15
    # every function reaches some prisms and leaves others
    sf = G.ring_scale(t.pos, t.conn, o.fns[1])
    assert 0 < np.isnan(sf).sum() < t.n_elems
    relz = o.state["relz"]
    assert 0 < (relz <= 0.6).sum() < t.n_elems


def test_ring_scale_in_single_precision():
    t = mesh.config_tiny(seed=5, n=6, n_layers=2)
    fn = dict(cx=12.3, cy=7.7, rin=3.0, rout=11.0)
    sf = G.ring_scale(t.pos, t.conn, fn)
    c = G.centres(t.pos, t.conn)
    d = np.hypot(c[:, 0] - 12.3, c[:, 1] - 7.7)
    inside = ~np.isnan(sf)
    assert ((d > 3.0) & (d < 11.0) == inside).all()
    # linear from 1 at the inner radius to 0 at the outer one, to float precision
    assert np.abs(sf[inside] - (1.0 - (d[inside] - 3.0) / 8.0)).max() < 1e-6


@ref_only
def test_mixed_functions_match_the_reference_driver():
    t, fns = G.mixed_case()
    R = Ref(t)
    G.add_functions(R, fns)
    o = G.GrowthOracle(t.pos, t.conn, t.node_placement)
    G.add_functions(o, fns)
    moved = t.pos + np.random.default_rng(3).uniform(-0.3, 0.3, size=t.pos.shape)
    R.set_positions(moved)
    for time in (0.0, 60.0):
        R.time = time
        F0 = R.get_Fg()[0]
        R.grow(60.0, t.rates)
        F1 = R.get_Fg()[0]
        Fo = o.grow(F0.reshape(-1, 3, 3), moved, time, 60.0, t.rates)
        assert np.abs(F1.reshape(-1, 3, 3) - Fo).max() <= 1e-15
    # without functions nothing grows (the reference keeps each prism's last
    # growth rotation, which turns the identity increment to within rounding)
    R.clear_growth_functions()
    F0 = R.get_Fg()[0]
    R.grow(60.0, np.zeros(3 * t.n_elems))
    assert np.abs(R.get_Fg()[0] - F0).max() <= 1e-15
    R.close()


def _rotated(t, degrees):
    """Current positions of the tissue turned by `degrees` about z."""
    a = math.radians(degrees)
    p = t.pos.reshape(-1, 3)
    q = p.copy()
    q[:, 0] = math.cos(a) * p[:, 0] - math.sin(a) * p[:, 1]
    q[:, 1] = math.sin(a) * p[:, 0] + math.cos(a) * p[:, 1]
    return q.reshape(-1)


def test_growth_turns_with_the_prism():
    """A sheet turned by 5 degrees: every prism's growth increment is turned
    by the angle the reference extracts (atan2(R01, R00) = -5 degrees); by
    0.5 degrees: below the reference's 0.017 thresholds, no turn."""
    t = mesh.config_tiny(seed=7, n=5, n_layers=2)
    o = G.GrowthOracle(t.pos, t.conn, t.node_placement)
    rot, Rz = G.growth_rotations(_rotated(t, 5.0), t.conn, o.inv_dXde)
    assert rot.all()
    np.testing.assert_allclose(np.arctan2(Rz[:, 1, 0], Rz[:, 0, 0]), math.radians(-5.0), atol=1e-12)
    rot, _ = G.growth_rotations(_rotated(t, 0.5), t.conn, o.inv_dXde)
    assert not rot.any()
    o.add_uniform_growth([4e-5, 1e-5, 0.0])
    F = o.grow(np.eye(3), _rotated(t, 5.0), 0.0, 60.0)
    d = np.exp(np.array([4e-5, 1e-5, 0.0]) * 60.0)
    c, s = math.cos(math.radians(-5.0)), math.sin(math.radians(-5.0))
    Rm = np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])
    np.testing.assert_allclose(F, np.broadcast_to(Rm @ np.diag(d) @ Rm.T, F.shape), atol=1e-12)


@ref_only
@pytest.mark.parametrize("degrees", [5.0, 0.5, -30.0])
def test_growth_rotation_matches_the_reference_driver(degrees):
    t = mesh.config_tiny(seed=8, n=5, n_layers=2)
    ra, aa = mesh.grid_growth_inputs(60, 4, 4)
    fns = [dict(kind="uniform", rates=[4e-5, 1e-5, 2e-6], angle_rad=0.3), dict(kind="grid", rates=ra, angles_deg=aa)]
    R = Ref(t)
    G.add_functions(R, fns)
    o = G.GrowthOracle(t.pos, t.conn, t.node_placement)
    G.add_functions(o, fns)
    turned = _rotated(t, degrees)
    R.set_positions(turned)
    F0 = R.get_Fg()[0]
    R.grow(60.0, t.rates)
    F1 = R.get_Fg()[0]
    Fo = o.grow(F0.reshape(-1, 3, 3), turned, 0.0, 60.0, t.rates)
    assert np.abs(F1.reshape(-1, 3, 3) - Fo).max() <= 1e-15
    R.close()


def test_rotated_fixture_matches_the_oracle():
    f = np.load(os.path.join(GOLD, G.ROTATED_FIXTURE + ".npz"))
    t, start, fns = G.rotated_case()
    o = G.GrowthOracle(t.pos, t.conn, t.node_placement)
    G.add_functions(o, fns)
    rot, _ = G.growth_rotations(start, t.conn, o.inv_dXde)
    assert rot.all()
    Fg = o.grow(np.eye(3), start, 0.0, t.dt, t.rates)
    assert np.abs(Fg.reshape(-1) - f["Fg_grow"]).max() <= 1e-15
    # without the turn the increment would differ
    Fu = G.GrowthOracle(t.pos, t.conn, t.node_placement)
    G.add_functions(Fu, fns)
    assert np.abs(Fu.grow(np.eye(3), t.pos, 0.0, t.dt, t.rates).reshape(-1) - f["Fg_grow"]).max() > 1e-4


@ref_only
def test_edge_cases_match_the_reference_driver():
    t = mesh.config_tiny(seed=35, n=6, n_layers=3)
    r2 = np.array([[[3e-5, 1e-5, 0.0], [1e-5, 3e-5, 0.0]], [[2e-5, 2e-5, 1e-6], [4e-5, 1e-5, 0.0]]])
    fns = [dict(kind="grid", rates=r2),
           dict(kind="uniform", rates=[5e-5, 0.0, 0.0], zmin=0.8, zmax=0.2),
           dict(kind="uniform", rates=[5e-5, 5e-5, 0.0], init_time=100.0, end_time=100.0),
           dict(kind="ring", centre=(12.0, 12.0), inner_radius=0.0, outer_radius=1e4, rates=[1e-5, 2e-5, 0.0],
                angle_rad=1.2)]
    start = G.turned(t.pos, 3.0)
    R = Ref(t)
    G.add_functions(R, fns)
    R.set_positions(start)
    R.time = 100.0
    F0 = R.get_Fg()[0]
    R.grow(60.0, np.zeros(3 * t.n_elems))
    F1 = R.get_Fg()[0]
    o = G.GrowthOracle(t.pos, t.conn, t.node_placement)
    G.add_functions(o, fns)
    Fo = o.grow(F0.reshape(-1, 3, 3), start, 100.0, 60.0, np.zeros(3 * t.n_elems))
    assert np.abs(F1.reshape(-1, 3, 3) - Fo).max() <= 1e-15
    R.close()


@pytest.mark.parametrize("label,kind,value,expect", G.TURN_THRESHOLD_CASES)
def test_turn_thresholds(label, kind, value, expect):
    """Start shapes whose distance 2|F - I| and rotation entries sit just
    below and just above the reference's 0.017: the prisms are turned exactly
    where the rotation's off-diagonal entries and angle exceed it."""
    t = mesh.config_tiny(seed=41, n=5, n_layers=2, jitter=0.0)
    o = G.GrowthOracle(t.pos, t.conn, t.node_placement)
    rot, Rz = G.growth_rotations(G.threshold_start(t, kind, value), t.conn, o.inv_dXde)
    assert (rot == expect).all(), label
    if expect:
        np.testing.assert_allclose(np.arctan2(Rz[:, 1, 0], Rz[:, 0, 0]), -value, atol=1e-12)


@ref_only
@pytest.mark.parametrize("label,kind,value,expect", G.TURN_THRESHOLD_CASES)
def test_turn_thresholds_match_the_reference_driver(label, kind, value, expect):
    t = mesh.config_tiny(seed=41, n=5, n_layers=2, jitter=0.0)
    fns = [dict(kind="uniform", rates=[5e-5, 1e-5, 0.0], angle_rad=0.3)]
    start = G.threshold_start(t, kind, value)
    R = Ref(t)
    G.add_functions(R, fns)
    R.set_positions(start)
    R.grow(60.0, np.zeros(3 * t.n_elems))
    F1 = R.get_Fg()[0]
    R.close()
    o = G.GrowthOracle(t.pos, t.conn, t.node_placement)
    G.add_functions(o, fns)
    Fo = o.grow(np.eye(3), start, 0.0, 60.0)
    assert np.abs(F1.reshape(-1, 3, 3) - Fo).max() <= 1e-15, label
    # the turn changes the increment well above that agreement
    Fu = G.GrowthOracle(t.pos, t.conn, t.node_placement)
    G.add_functions(Fu, fns)
    moved = np.abs(Fu.grow(np.eye(3), t.pos, 0.0, 60.0) - Fo).max()
    assert (moved > 1e-7) == expect, (label, moved)
