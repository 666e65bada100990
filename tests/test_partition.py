"""One mesh over two ranks (tissuefolding_paperversion_gb300.partition): the
z-column strip partition, the one-shot assembly halo and the per-product
solve halo of the distributed Krylov solve, run as two gloo ranks on CPU.
The oracle's element evaluation on each rank's submesh stands in for a GPU
per rank; the assembled owned rows of A = K^T, the right-hand side and the
solution of A du = g must reproduce the one-process assembly and solve."""
import os
import socket

import numpy as np
import pytest

from tissuefolding_paperversion_gb300 import mesh, partition


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _case():
    t = mesh.config_tiny(seed=91, n=9, n_layers=3, eta=100.0)
    Fg = mesh.growth_Fg(t, seed=92, amp=0.03)
    uk, un = mesh.perturbed_state(t, seed=93, amp=0.1)
    return t, Fg, uk, un


def test_strips_keep_columns_whole_and_balance_prisms():
    t, _, _, _ = _case()
    for n in (1, 2, 3, 4):
        part = partition.StripPartition(t.pos, t.conn, n)
        cxy = np.round(t.pos.reshape(-1, 3)[t.conn.reshape(-1, 6)].mean(axis=1)[:, :2], 9)
        _, col = np.unique(cxy, axis=0, return_inverse=True)
        for c in np.unique(col):
            assert np.unique(part.elem_part[col.reshape(-1) == c]).size == 1
        counts = np.bincount(part.elem_part, minlength=n)
        layers = 3
        assert counts.min() > 0 and counts.max() - counts.min() <= 2 * (t.n_elems // layers) // n + layers
        owned = np.concatenate([R["owned"] for R in part.ranks])
        assert np.array_equal(np.sort(owned), np.arange(t.n_nodes))
        for r, R in enumerate(part.ranks):
            assert np.all(part.node_owner[R["spmv_ghosts"]] != r)
            assert np.all(part.node_owner[R["asm_ghosts"]] != r)
    with pytest.raises(ValueError):
        partition.StripPartition(t.pos, t.conn, 0)


def _rank_main(rank, world, port, out_path):
    import torch.distributed as dist

    from oracle.oracle import CLOSED, Port

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t, Fg, uk, un = _case()
        part = partition.StripPartition(t.pos, t.conn, world)
        sub, nodes = part.submesh(t, rank)
        e = part.ranks[rank]["elems"]
        n3 = (3 * nodes[:, None] + np.arange(3)[None, :]).reshape(-1)
        p = Port(sub)
        p.set_Fg(Fg.reshape(-1, 9)[e].reshape(-1))
        p.set_positions(un[n3])
        area = p.update_viscosity_surfaces()
        ev = p.element_eval(uk[n3], un[n3], t.dt, CLOSED)
        vel = (uk[n3] - un[n3]) * (1.0 / t.dt)
        rs = partition.RankSystem(part, rank, partition.Comm(dist))
        A, g = rs.assemble(nodes, ev["Ke"], ev["Kv"], ev["fe"], ev["fv"], area, vel, t.dt, t.ext_visc, t.fixed)
        du, it, rr = rs.bicgstab(rtol=1e-12)
        np.savez(out_path.format(rank), owned=rs.owned, cols=rs.cols, A=A.toarray(), g=g, du=du, iters=it, rr=rr)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reproduce_the_one_process_assembly_and_solve(tmp_path):
    pytest.importorskip("torch")
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla
    import torch.multiprocessing as mp

    from oracle.oracle import CLOSED, Port, build_port

    build_port()
    out = str(tmp_path / "rank{}.npz")
    mp.start_processes(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    t, Fg, uk, un = _case()
    p = Port(t)
    p.set_Fg(Fg)
    p.set_positions(un)
    p.update_viscosity_surfaces()
    p.assemble(uk, un, t.dt, CLOSED)
    ia, ja = p.structure()
    a, g = p.values()
    n = 3 * t.n_nodes
    K = sp.csr_matrix((a, ja, ia), shape=(n, n))
    A = K.T.tocsr()
    du = sla.spsolve(A.tocsc(), g)
    seen = np.zeros(t.n_nodes, dtype=bool)
    for r in range(2):
        f = np.load(out.format(r))
        own3 = (3 * f["owned"][:, None] + np.arange(3)[None, :]).reshape(-1)
        col3 = (3 * f["cols"][:, None] + np.arange(3)[None, :]).reshape(-1)
        Aref = A[own3][:, col3].toarray()
        assert np.abs(f["A"] - Aref).max() <= 1e-13 * np.abs(Aref).max(), r
        # every nonzero of the owned rows lies in the rank's owned and ghost columns
        assert np.isclose(np.abs(A[own3]).sum(), np.abs(Aref).sum(), rtol=1e-13)
        assert np.abs(f["g"] - g[own3]).max() <= 1e-13 * np.abs(g).max(), r
        assert float(f["rr"]) <= 1e-12 and int(f["iters"]) > 0
        assert np.abs(f["du"] - du[own3]).max() <= 1e-9 * np.abs(du).max(), r
        seen[f["owned"]] = True
    assert seen.all()
