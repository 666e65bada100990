"""The CPU oracle (oracle/tf_oracle.c), pinned against the reference.

* against the golden fixtures made by tests/golden/make_golden.py from the
  reference's own sources (runs everywhere);
* against oracle/_ref live, bit for bit (only where the reference checkout is
  present);
* properties the reference's maths implies: the closed-form tangent equals
  the literal 3^6 contraction, the tangent is the derivative of the residual,
  rigid motions cause no force, the elastic tangent is symmetric.
"""
import os

import numpy as np
import pytest

from oracle.oracle import CLOSED, LITERAL, Port, Ref
from tissuefolding_paperversion_gb300 import mesh

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _load(name):
    path = os.path.join(GOLD, name + ".npz")
    if not os.path.exists(path):
        pytest.fail(f"missing golden fixture {path}; run tests/golden/make_golden.py")
    return np.load(path)


def _rel(a, b):
    s = np.abs(b).max()
    return np.abs(a - b).max() / (s if s > 0 else 1.0)


@pytest.mark.parametrize("name,eta,seed", [("elem_tiny_elastic", 0.0, 11), ("elem_tiny_viscous", 100.0, 12)])
def test_port_matches_reference_element_fixture(name, eta, seed):
    f = _load(name)
    t = mesh.config_tiny(seed=seed, n=3, n_layers=2, eta=eta)
    p = Port(t)
    p.set_Fg(f["Fg"])
    ev = p.element_eval(f["uk"], f["un"], float(f["dt"]), LITERAL)
    for k in ("Ke", "Kv", "fe", "fv"):
        assert _rel(ev[k], f[k]) <= 1e-14, k
    p.set_positions(f["uk"])
    area = p.update_viscosity_surfaces()
    assert _rel(area, f["area"]) <= 1e-15
    p.assemble(f["uk"], f["un"], float(f["dt"]), LITERAL)
    ia, ja, a = p.export_filtered(1e-13)
    _, g = p.values()
    # the value-filtered pattern is integer data: bit-exact
    assert np.array_equal(ia, f["ia"]) and np.array_equal(ja, f["ja"])
    assert _rel(a, f["a"]) <= 1e-14
    assert _rel(g, f["g"]) <= 1e-14


@pytest.mark.parametrize("name,seed,eta", [("steps_tiny_elastic", 13, 0.0), ("steps_tiny_viscous", 14, 100.0)])
def test_port_matches_reference_newton_steps(name, seed, eta):
    f = _load(name)
    t = mesh.config_tiny(seed=seed, n=4, n_layers=2, eta=eta)
    p = Port(t)
    for s in range(f["positions"].shape[0]):
        out = p.step(t.dt, t.rates, LITERAL)
        assert out["iters"] == f["iters"][s]
        assert _rel(p.positions(), f["positions"][s]) <= 1e-13


def test_port_matches_reference_small_config_20_steps():
    f = _load("steps_small")
    t = mesh.config_small(seed=0)
    p = Port(t)
    for s in range(f["positions"].shape[0]):
        out = p.step(t.dt, t.rates, CLOSED)
        ref = f["positions"][s]
        assert np.abs(p.positions() - ref).max() <= 1e-8 * np.abs(ref).max(), s
        assert out["iters"] == f["iters"][s]


@pytest.mark.skipif(not Ref.available(), reason="reference checkout not present")
@pytest.mark.parametrize("eta", [0.0, 100.0])
def test_port_bit_exact_against_live_reference(eta):
    t = mesh.config_tiny(seed=21, n=5, n_layers=3, eta=eta)
    p, r = Port(t), Ref(t)
    Fg = mesh.growth_Fg(t, seed=5)
    p.set_Fg(Fg)
    r.set_Fg(Fg)
    uk, un = mesh.perturbed_state(t, seed=6)
    a = p.element_eval(uk, un, t.dt, LITERAL)
    b = r.element_eval(uk, un, t.dt)
    for k in ("Ke", "Kv", "fe", "fv"):
        assert np.array_equal(a[k], b[k]), k
    # the reference's element evaluation moves its nodes to uk; restart both
    p.set_positions(t.pos)
    r.set_positions(t.pos)
    for _ in range(2):
        p.step(t.dt, t.rates, LITERAL)
        r.step(t.dt, t.rates)
        assert np.array_equal(p.positions(), r.positions())


def test_closed_form_equals_literal():
    t = mesh.config_tiny(seed=31, n=4, n_layers=2, eta=50.0)
    p = Port(t)
    p.set_Fg(mesh.growth_Fg(t, seed=32, amp=0.05))
    uk, un = mesh.perturbed_state(t, seed=33, amp=0.3)
    a = p.element_eval(uk, un, t.dt, LITERAL)
    b = p.element_eval(uk, un, t.dt, CLOSED)
    assert _rel(b["Ke"], a["Ke"]) <= 1e-12
    assert np.array_equal(a["Kv"], b["Kv"]) and np.array_equal(a["fe"], b["fe"])


def test_tangent_is_derivative_of_residual():
    # K as stored by the reference satisfies K^T = -dg/du (it solves K^T du = g).
    t = mesh.config_tiny(seed=41, n=3, n_layers=2, eta=80.0)
    t.fixed[:] = 0
    p = Port(t)
    p.set_Fg(mesh.growth_Fg(t, seed=42))
    uk, un = mesh.perturbed_state(t, seed=43)
    p.set_positions(un)
    p.update_viscosity_surfaces()
    p.assemble(uk, un, t.dt, CLOSED)
    ia, ja = p.structure()
    a, _ = p.values()
    n = 3 * t.n_nodes
    K = np.zeros((n, n))
    for r in range(n):
        K[r, ja[ia[r]:ia[r + 1]]] = a[ia[r]:ia[r + 1]]
    h = 1e-6
    J = np.zeros((n, n))
    for j in range(n):
        e = np.zeros(n)
        e[j] = h
        J[:, j] = -(p.residual(uk + e, un, t.dt) - p.residual(uk - e, un, t.dt)) / (2 * h)
    assert _rel(J, K.T) <= 1e-6


def test_rigid_motion_gives_no_force():
    t = mesh.config_tiny(seed=51, n=4, n_layers=2, eta=0.0)
    t.fixed[:] = 0
    t.ext_visc[:] = 0.0
    p = Port(t)
    c, s = np.cos(0.3), np.sin(0.3)
    R = np.array([[c, -s, 0], [s, c, 0], [0, 0, 1.0]])
    x = t.pos.reshape(-1, 3) @ R.T + np.array([3.0, -2.0, 1.0])
    g = p.residual(x.reshape(-1), x.reshape(-1), t.dt)
    assert np.abs(g).max() <= 1e-9


def test_elastic_tangent_symmetric():
    t = mesh.config_tiny(seed=61, n=4, n_layers=2, eta=0.0)
    p = Port(t)
    p.set_Fg(mesh.growth_Fg(t, seed=62))
    uk, un = mesh.perturbed_state(t, seed=63)
    ev = p.element_eval(uk, un, t.dt, LITERAL)
    Ke = ev["Ke"]
    assert _rel(Ke, np.transpose(Ke, (0, 2, 1))) <= 1e-12


def test_bound_fixture_moves_couples_together():
    """The binding fixture came from the reference's own solver: every slave
    DOF moved by exactly its master's displacement."""
    f = np.load(os.path.join(GOLD, "steps_tiny_bound.npz"))
    t = mesh.config_tiny(seed=15, n=5, n_layers=2, eta=100.0)
    d = f["positions"][-1] - t.pos
    np.testing.assert_allclose(d[f["slaves"]], d[f["masters"]], rtol=0, atol=1e-12)
    assert np.abs(d[f["slaves"]]).max() > 1e-3
