"""Parity of the CUDA path (through the C ABI) with the CPU oracle and the
reference's golden vectors.

Tolerances (FP64 throughout):
  * element tangents / forces and assembled K, g: 1e-11 relative to the
    largest entry (the GPU uses the exact closed form of the reference's
    3^6 contraction and atomics, so the last bits differ);
  * block pattern and the value-filtered CSR pattern: bit-exact;
  * node positions after every Newton step: 1e-8 relative.
"""
import os

import numpy as np
import pytest

from oracle.oracle import CLOSED, LITERAL, Port
from tissuefolding_paperversion_gb300 import api, mesh

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
TOL_K = 1e-11
TOL_POS = 1e-8


def _rel(a, b):
    s = np.abs(b).max()
    return np.abs(a - b).max() / (s if s > 0 else 1.0)


def _csr_dense(ia, ja, a, n):
    K = np.zeros((n, n))
    for r in range(n):
        K[r, ja[ia[r]:ia[r + 1]]] = a[ia[r]:ia[r + 1]]
    return K


@pytest.mark.parametrize("eta", [0.0, 100.0])
def test_element_tangent_and_forces_match_oracle(eta):
    t = mesh.config_tiny(seed=71, n=5, n_layers=3, eta=eta)
    Fg = mesh.growth_Fg(t, seed=72, amp=0.05)
    uk, un = mesh.perturbed_state(t, seed=73, amp=0.2)
    p = Port(t)
    p.set_Fg(Fg)
    ref = p.element_eval(uk, un, t.dt, LITERAL)
    with api.Solver(t) as s:
        s.set_Fg(Fg)
        s.set_state(uk, un, t.dt)
        got = s.element_eval()
    for k in ("Ke", "Kv", "fe", "fv"):
        assert _rel(got[k], ref[k]) <= TOL_K, k


@pytest.mark.parametrize("name,eta,seed", [("elem_tiny_elastic", 0.0, 11), ("elem_tiny_viscous", 100.0, 12)])
def test_element_and_assembly_match_reference_fixture(name, eta, seed):
    f = np.load(os.path.join(GOLD, name + ".npz"))
    t = mesh.config_tiny(seed=seed, n=3, n_layers=2, eta=eta)
    with api.Solver(t) as s:
        s.set_Fg(f["Fg"])
        s.set_state(f["uk"], f["un"], float(f["dt"]))
        got = s.element_eval()
        for k in ("Ke", "Kv", "fe", "fv"):
            assert _rel(got[k], f[k]) <= TOL_K, k
        s.set_positions(f["uk"])
        s.begin_step(float(f["dt"]))        # viscosity surfaces at uk; un := uk
        assert _rel(s.viscosity_surfaces(), f["area"]) <= 1e-14
        s.set_state(f["uk"], f["un"], float(f["dt"]))
        s.assemble()
        ia, ja, a = s.export_csr(1e-13)
        g = s.residual()
    assert np.array_equal(ia, f["ia"]) and np.array_equal(ja, f["ja"])
    assert _rel(a, f["a"]) <= TOL_K
    assert _rel(g, f["g"]) <= TOL_K


@pytest.mark.parametrize("eta,deterministic", [(0.0, False), (100.0, False), (100.0, True)])
def test_assembled_system_matches_oracle(eta, deterministic):
    t = mesh.config_small(seed=1)
    t.eta[:] = eta
    Fg = mesh.growth_Fg(t, seed=81, amp=0.01)
    uk, un = mesh.perturbed_state(t, seed=82, amp=0.1)
    p = Port(t)
    p.set_Fg(Fg)
    p.set_positions(un)
    area = p.update_viscosity_surfaces()
    p.assemble(uk, un, t.dt, CLOSED)
    ia0, ja0, a0 = p.export_filtered(1e-13)
    _, g0 = p.values()
    with api.Solver(t, deterministic=deterministic) as s:
        s.set_Fg(Fg)
        s.set_state(uk, un, t.dt)
        s.set_viscosity_surfaces(area)
        s.assemble()
        ia, ja, a = s.export_csr(1e-13)
        g = s.residual()
    assert np.array_equal(ia, ia0) and np.array_equal(ja, ja0)
    assert _rel(a, a0) <= TOL_K
    assert _rel(g, g0) <= TOL_K


def test_linear_solve_is_the_transposed_system():
    t = mesh.config_tiny(seed=91, n=5, n_layers=2, eta=100.0)
    uk, un = mesh.perturbed_state(t, seed=92)
    p = Port(t)
    p.set_positions(un)
    area = p.update_viscosity_surfaces()
    p.assemble(uk, un, t.dt, CLOSED)
    du_ref = p.solve()
    with api.Solver(t, krylov_rtol=1e-13) as s:
        s.set_state(uk, un, t.dt)
        s.set_viscosity_surfaces(area)
        s.assemble()
        out = s.solve()
        du = s.delta_u()
        ia, ja, a = s.export_csr(0.0)
        g = s.residual()
    K = _csr_dense(ia, ja, a, 3 * t.n_nodes)
    assert np.abs(K.T @ du - g).max() <= 1e-9 * np.abs(g).max()
    assert _rel(du, du_ref) <= 1e-9
    assert out["relres"] <= 1e-13


def _run_steps_against(fixture, t, tol):
    f = np.load(os.path.join(GOLD, fixture + ".npz"))
    with api.Solver(t) as s:
        s.set_growth_rates(t.rates)
        for k in range(f["positions"].shape[0]):
            out = s.newton_step(t.dt, allow_not_converged=False)
            ref = f["positions"][k]
            pos = s.positions()
            assert np.abs(pos - ref).max() <= tol * np.abs(ref).max(), (k, np.abs(pos - ref).max())
            assert out["iters"] == f["iters"][k], (k, out["iters"])
        Fg, _ = s.get_Fg()
    assert _rel(Fg, f["Fg"]) <= 1e-13


def test_newton_steps_match_reference_small_config():
    _run_steps_against("steps_small", mesh.config_small(seed=0), TOL_POS)


@pytest.mark.parametrize("name,seed,eta", [("steps_tiny_elastic", 13, 0.0), ("steps_tiny_viscous", 14, 100.0)])
def test_newton_steps_match_reference_tiny(name, seed, eta):
    _run_steps_against(name, mesh.config_tiny(seed=seed, n=4, n_layers=2, eta=eta), TOL_POS)


def test_deterministic_assembly_is_bitwise_reproducible():
    t = mesh.config_small(seed=2)
    t.eta[:] = 50.0
    uk, un = mesh.perturbed_state(t, seed=3, amp=0.1)
    outs = []
    for _ in range(2):
        with api.Solver(t, deterministic=True) as s:
            s.set_state(uk, un, t.dt)
            s.assemble()
            outs.append((s.export_csr(0.0)[2], s.residual()))
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def _force_scale(t):
    """Force a unit strain produces on one element face: max E times the mean
    squared in-plane spacing.  Element forces of nearly unstressed elements
    are tiny, so they are compared at this scale; FP64 evaluation at
    coordinates ~1000 um carries strain noise ~1e-13 in the reference too."""
    p = t.pos.reshape(-1, 3)
    c = t.conn.reshape(-1, 6)
    h2 = np.mean(np.sum((p[c[:, 1]] - p[c[:, 0]]) ** 2, axis=1))
    return float(np.max(t.E)) * h2


def test_large_mesh_sampled_elements_and_residual():
    """Full-size mesh (320k prisms): size-independent checks against the oracle."""
    t = mesh.config_large(seed=0)
    with api.Solver(t) as s:
        s.set_growth_rates(t.rates)
        out = s.newton_step(t.dt, allow_not_converged=False)
        assert out["converged"] and out["dunorm"][-1] <= 1e-8
        pos = s.positions()
        Fg, _ = s.get_Fg()
        un = t.pos
        # residual of the GPU's converged state, evaluated by both sides
        s.set_state(pos, un, t.dt)
        s.assemble()
        g_gpu = s.residual()
        area = s.viscosity_surfaces()
        rng = np.random.default_rng(0)
        sample = np.sort(rng.choice(t.n_elems, 64, replace=False))
        got = [s.element_eval(int(e), 1) for e in sample]
    p = Port(t)
    p.set_Fg(Fg)
    p.set_viscosity_surfaces(area)
    g_cpu = p.residual(pos, un, t.dt)
    fs = _force_scale(t)
    assert np.abs(g_gpu - g_cpu).max() <= 1e-11 * fs
    # the GPU's converged state is an equilibrium of the oracle's physics
    assert np.abs(g_cpu).max() <= 1e-8 * fs
    for e, r in zip(sample, got):
        ref = p.element_eval(pos, un, t.dt, LITERAL, int(e), 1)
        for k in ("Ke", "Kv"):
            assert _rel(r[k], ref[k]) <= TOL_K, (e, k)
        for k in ("fe", "fv"):
            assert np.abs(r[k] - ref[k]).max() <= 1e-11 * fs, (e, k)
