"""tf_add_K_triplets: entries written into K after the assembly (the hook of
the reference's packing / myosin writers, which add to NRSolver->K between the
element assembly and calcutateFixedK), inside and outside the element pattern."""
import numpy as np
import pytest

from tissuefolding_paperversion_gb300 import api, mesh

pytestmark = pytest.mark.gpu


def _dense(ia, ja, a, n):
    K = np.zeros((n, n))
    for r in range(n):
        K[r, ja[ia[r]:ia[r + 1]]] = a[ia[r]:ia[r + 1]]
    return K


def test_triplets_in_and_outside_the_pattern():
    t = mesh.config_tiny(seed=31, n=5, n_layers=2, eta=100.0)
    uk, un = mesh.perturbed_state(t, seed=32, amp=0.05)
    n3 = 3 * t.n_nodes
    free = np.flatnonzero(t.fixed == 0)
    fixed = np.flatnonzero(t.fixed != 0)
    pos = t.pos.reshape(-1, 3)
    # two far-apart apical nodes: not element neighbours
    ap = np.flatnonzero(t.node_placement == 1)
    a0 = ap[np.argmin(pos[ap, 0] + pos[ap, 1])]
    a1 = ap[np.argmax(pos[ap, 0] + pos[ap, 1])]
    rows = [3 * a0, 3 * a0 + 1, 3 * a1 + 2, 3 * a0, free[5], fixed[0], free[7]]
    cols = [3 * a1, 3 * a1 + 2, 3 * a0, 3 * a0, free[5], free[3], fixed[1]]
    vals = [1.5, -2.0, 0.75, 3.0, 4.0, 9.0, 9.0]
    with api.Solver(t, krylov_rtol=1e-12) as s:
        s.set_positions(un)
        s.begin_step(t.dt)
        s.set_state(uk, un, t.dt)
        s.assemble()
        K0 = _dense(*s.export_csr(0.0), n3)
        s.add_K_triplets(rows[:3], cols[:3], vals[:3])
        s.add_K_triplets(rows[3:], cols[3:], vals[3:])
        K1 = _dense(*s.export_csr(0.0), n3)
        g = s.residual()
        out = s.solve()
        du = s.delta_u()
        s.assemble()                 # a new assembly clears the added values
        K2 = _dense(*s.export_csr(0.0), n3)
    want = K0.copy()
    for r, c, v in zip(rows, cols, vals):
        if t.fixed[r] or t.fixed[c]:
            continue                 # dropped, as calcutateFixedK would zero them
        want[r, c] += v
    assert K0[3 * a0, 3 * a1] == 0.0          # the far pair is outside the pattern
    np.testing.assert_allclose(K1, want, rtol=0, atol=1e-12 * np.abs(K0).max())
    # the linear solve uses the added entries: K^T du = g
    assert out["relres"] <= 1e-12
    assert np.abs(K1.T @ du - g).max() <= 1e-9 * np.abs(g).max()
    # (the atomic scatter reorders the element sums: last-bit differences)
    np.testing.assert_allclose(K2, K0, rtol=0, atol=1e-13 * np.abs(K0).max())


def test_triplets_need_an_assembly_and_valid_indices():
    t = mesh.config_tiny(seed=33, n=4, n_layers=2)
    with api.Solver(t) as s:
        with pytest.raises(api.TfError):
            s.add_K_triplets([0], [0], [1.0])
        s.assemble()
        with pytest.raises(api.TfError):
            s.add_K_triplets([3 * t.n_nodes], [0], [1.0])
