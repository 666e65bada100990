"""Implicit packing between tissue surfaces on the GPU (tf_set_packing)
against fixtures the reference's own classes produced (tests/golden/
make_golden.py --only-packing) and against the packing restatement
(oracle/packing.py): couple detection, node masses, the assembled system with
the packing forces and Jacobian, Newton steps with couples re-detected at every
step, and larger sheets where the hashed cell list must find exactly the
couples of the O(N^2) scan."""
import os

import numpy as np
import pytest

from oracle import packing as op
from tissuefolding_paperversion_gb300 import api, mesh

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
CASES = [("steps_facing_packing", dict(seed=12, gap=1.5, E=100000.0, eta=0.0)),
         ("steps_facing_packing_viscous", dict(seed=13, gap=1.5, E=100000.0, eta=100.0))]
TOL_POS = 1e-8
TOL_K = 1e-11


def _dense(ia, ja, a, n):
    K = np.zeros((n, n))
    for r in range(n):
        K[r, ja[ia[r]:ia[r + 1]]] = a[ia[r]:ia[r + 1]]
    return K


@pytest.mark.parametrize("name,kw", CASES)
def test_detection_and_assembled_system_match_the_reference(name, kw):
    f = np.load(os.path.join(GOLD, name + ".npz"))
    t = mesh.config_facing_sheets(**kw)
    uk, un = mesh.perturbed_state(t, seed=7, amp=0.05)
    n3 = 3 * t.n_nodes
    with api.Solver(t, deterministic=True) as s:
        s.set_packing(True, reference_merge=bool(f["drop_last_segment"]))
        s.set_positions(un)
        s.begin_step(t.dt)
        pk = s.packing()
        np.testing.assert_array_equal(pk["nodes"], f["asm_nodes"])
        np.testing.assert_allclose(pk["w"], f["asm_w"], rtol=0, atol=1e-15)
        np.testing.assert_allclose(pk["mbar"], f["asm_mbar"], rtol=1e-14)
        np.testing.assert_allclose(s.packing_masses(), f["asm_masses"], rtol=1e-14)
        assert abs(pk["threshold"] - float(f["asm_threshold"])) <= 1e-14 * float(f["asm_threshold"])
        s.set_state(uk, un, t.dt)
        s.assemble()
        K = _dense(*s.export_csr(0.0), n3)
        g = s.residual()
    Kr = _dense(f["asm_ia"], f["asm_ja"], f["asm_a"], n3)
    scale = np.abs(Kr).max()
    assert np.abs(K - Kr).max() <= TOL_K * scale, np.abs(K - Kr).max() / scale
    gr = f["asm_g"]
    assert np.abs(g - gr).max() <= TOL_K * np.abs(gr).max()
    # the couples' off-diagonal blocks are outside the element pattern
    a, b = f["asm_nodes"][0]
    assert K[3 * a, 3 * b] != 0.0


@pytest.mark.parametrize("name,kw", CASES)
@pytest.mark.parametrize("precond", [1, 2])
def test_newton_steps_with_packing_match_the_reference(name, kw, precond):
    # precond 2: the multigrid's coarse levels carry the couples' blocks as
    # P^T X P (the element graph never joins the two sheets)
    f = np.load(os.path.join(GOLD, name + ".npz"))
    t = mesh.config_facing_sheets(**kw)
    off = np.concatenate([[0], np.cumsum(f["pk_n"])])
    # order-fixed assembly: block-Jacobi BiCGStab at 1e-12 on these stiff
    # contact systems is sensitive to the summation order of the atomic
    # scatter (3,900-5,300 iterations over the two steps from run to run, and
    # once in a while a Newton iteration more); with the order fixed every run
    # takes the same path
    with api.Solver(t, krylov_rtol=1e-12, precond=precond, deterministic=True) as s:
        s.set_growth_rates(t.rates)
        s.set_packing(True, reference_merge=bool(f["drop_last_segment"]))
        for k in range(f["positions"].shape[0]):
            out = s.newton_step(t.dt, allow_not_converged=False)
            pk = s.packing()
            np.testing.assert_array_equal(pk["nodes"], f["pk_nodes"][off[k]:off[k + 1]])
            ref = f["positions"][k]
            pos = s.positions()
            assert np.abs(pos - ref).max() <= TOL_POS * np.abs(ref).max(), (k, np.abs(pos - ref).max())
            assert out["iters"] == f["iters"][k], (k, out["iters"], f["iters"][k])


@pytest.mark.parametrize("seed,n,merge", [(3, 12, True), (4, 20, False), (6, 31, True)])
def test_cell_list_finds_the_couples_of_the_full_scan(seed, n, merge):
    t = mesh.config_facing_sheets(seed=seed, n=n, gap=1.5, E=100000.0, offset=(1.3, -0.7))
    vref = op.reference_volumes(t.pos.reshape(-1, 3)[t.conn.reshape(-1, 6)])
    m = op.node_masses(t.conn, t.n_nodes, vref, np.tile(np.eye(3), (t.n_elems, 1, 1)))
    want = op.detect(t.pos, t.conn, t.node_placement, m, merge)
    with api.Solver(t) as s:
        s.set_packing(True, reference_merge=merge)
        s.begin_step(t.dt)
        got = s.packing()
        np.testing.assert_allclose(s.packing_masses(), m, rtol=1e-14)
    assert len(want["nodes"]) > 0
    np.testing.assert_array_equal(got["nodes"], want["nodes"])
    np.testing.assert_allclose(got["w"], want["w"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(got["mbar"], want["mbar"], rtol=1e-14)
    assert abs(got["threshold"] - want["threshold"]) <= 1e-13 * want["threshold"]


@pytest.mark.parametrize("seed,n", [(8, 9), (9, 40)])
def test_reference_box_when_node_0_holds_the_maximum(seed, n):
    """Node 0 alone at the largest x: the device box replays the reference's
    running minimum, so the couples are the reference's."""
    t = mesh.config_facing_sheets(seed=seed, n=n, gap=1.5, E=100000.0, offset=(0.4, 0.2))
    t = mesh.swap_nodes(t, 0, int(np.argmax(t.pos.reshape(-1, 3)[:, 0])))
    t.pos[0] += 0.3
    vref = op.reference_volumes(t.pos.reshape(-1, 3)[t.conn.reshape(-1, 6)])
    m = op.node_masses(t.conn, t.n_nodes, vref, np.tile(np.eye(3), (t.n_elems, 1, 1)))
    want = op.detect(t.pos, t.conn, t.node_placement, m, True)
    with api.Solver(t) as s:
        s.set_packing(True, reference_merge=True)
        s.begin_step(t.dt)
        got = s.packing()
    assert len(want["nodes"]) > 0
    np.testing.assert_array_equal(got["nodes"], want["nodes"])
    np.testing.assert_allclose(got["w"], want["w"], rtol=0, atol=1e-15)


def test_multigrid_sees_the_couples():
    # without the couples' coarse images the V-cycle's coarse correction misses
    # the stiff coupling between the sheets and the solve diverges; with them
    # it needs a fraction of block-Jacobi's iterations
    t = mesh.config_facing_sheets(seed=12, gap=1.5, E=100000.0)
    tot = {}
    for pc in (1, 2):
        with api.Solver(t, precond=pc) as s:
            s.set_growth_rates(t.rates)
            s.set_packing(True)
            tot[pc] = sum(s.newton_step(t.dt, allow_not_converged=False)["krylov_total"] for _ in range(2))
            if pc == 2:
                assert s.multigrid_info()[0]
    assert 3 * tot[2] < tot[1], tot


def test_packing_is_bitwise_reproducible_and_switches_off():
    t = mesh.config_facing_sheets(seed=12, gap=1.5, E=100000.0)
    runs = []
    for _ in range(2):
        with api.Solver(t, deterministic=True) as s:
            s.set_growth_rates(t.rates)
            s.set_packing(True)
            its = [s.newton_step(t.dt)["iters"] for _ in range(2)]
            runs.append((s.positions(), its))
    assert np.array_equal(runs[0][0], runs[1][0]) and runs[0][1] == runs[1][1]
    # switched off again: the same steps as a solver that never packed
    with api.Solver(t, deterministic=True) as s, api.Solver(t, deterministic=True) as s0:
        for x in (s, s0):
            x.set_growth_rates(t.rates)
        s.set_packing(True)
        s.set_packing(False)
        s.newton_step(t.dt)
        s0.newton_step(t.dt)
        assert np.array_equal(s.positions(), s0.positions())
        assert s.packing()["nodes"].shape == (0, 2)


def test_triplets_add_on_top_of_the_packing_jacobian():
    t = mesh.config_facing_sheets(seed=12, gap=1.5, E=100000.0)
    n3 = 3 * t.n_nodes
    with api.Solver(t) as s:
        s.set_packing(True)
        s.begin_step(t.dt)
        s.assemble()
        K0 = _dense(*s.export_csr(0.0), n3)
        a, b = s.packing()["nodes"][0]
        free = [q for q in range(3) if t.fixed[3 * a + q] == 0 and t.fixed[3 * b + q] == 0]
        r, c = 3 * a + free[0], 3 * b + free[0]
        s.add_K_triplets([r, c], [c, r], [2.5, -1.0])
        K1 = _dense(*s.export_csr(0.0), n3)
    D = K1 - K0
    assert D[r, c] == pytest.approx(2.5, rel=1e-12) and D[c, r] == pytest.approx(-1.0, rel=1e-12)
    D[r, c] = D[c, r] = 0.0
    assert np.abs(D).max() == 0.0


def test_packing_is_refused_where_it_is_not_defined():
    t = mesh.config_facing_sheets(seed=12, gap=1.5, E=100000.0)
    with api.Batch([t, t]) as bt:
        assert bt.L.tf_set_packing(bt.h, 1, 1) == api.TF_BAD_INPUT      # single-mesh handles only
    with api.Solver(t) as s:
        assert s.L.tf_set_packing(s.h, 1, 2) == api.TF_BAD_INPUT        # unknown flag
        s.set_packing(True)
        xy = t.pos.reshape(-1, 3)
        params = np.array([xy[:, 0].mean(), xy[:, 1].mean(), 10.0, 8.0])
        with pytest.raises(api.TfError):
            s.adjoint_forward(np.full(t.n_elems, 1e-5), np.log(t.E), 2, t.dt, 1, params)
