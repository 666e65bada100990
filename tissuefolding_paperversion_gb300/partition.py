"""One mesh over several ranks (one GPU each): z-column strips with an
interface halo.

The reference assembles and solves one mesh in one process
(NewtonRaphsonSolver::calculateForcesAndJacobianMatrixNR, an OpenMP loop over
prisms, NewtonRaphsonSolver.cpp:257-271, then one Pardiso solve, :418-683).
Over ranks the work splits like this:

* **elements**: prisms are grouped into columns (all layers above one
  triangle share their centroid's xy) and the columns are cut into strips of
  about equal prism count across the sheet's longer in-plane axis; a rank
  evaluates the prisms of its strip.  Because a column never straddles two
  ranks, apical and basal faces -- the viscosity surfaces -- are a rank's own.
* **rows**: every node is owned by the lowest rank among the prisms that
  touch it; a rank keeps the rows of A = K^T (the system the reference
  solves, Pardiso iparm[11] = 1) and of g for its owned nodes.
* **assembly halo** (once per assembly): a rank's prisms also produce entries
  in rows of nodes it does not own (the interface); those entries, their
  parts of g and of the node viscosity areas go to the owner, which adds
  them to its own -- after that every owned row is complete.
* **solve halo** (every matrix-vector product): a rank needs x at the
  neighbours of its owned nodes that other ranks own; the owners send them.
  Dot products are sums over owned entries plus one all-reduce.

The per-rank element work is any evaluator of the reference's element
quantities (18 x 18 Ke and Kv in the reference's orientation, 6 x 3 forces)
on the rank's submesh -- a GPU handle created on that submesh, or a CPU
evaluator -- and the per-rank Krylov recurrences are FP64 block-Jacobi
BiCGStab, as on one GPU.  Communication goes through torch.distributed
point-to-point sends and all-reduces (gloo on CPU ranks, NCCL on GPU ranks).
"""
from __future__ import annotations

import numpy as np


class StripPartition:
    """Z-column strips of a prism mesh over `n_parts` ranks."""

    def __init__(self, pos, conn, n_parts: int):
        if n_parts < 1:
            raise ValueError("the number of parts must be positive")
        p = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
        c = np.asarray(conn, dtype=np.int64).reshape(-1, 6)
        self.n_nodes, self.n_elems, self.n_parts = p.shape[0], c.shape[0], n_parts
        cxy = p[c].mean(axis=1)[:, :2]
        ext = cxy.max(axis=0) - cxy.min(axis=0) if self.n_elems else np.zeros(2)
        axis = int(ext[1] > ext[0])
        # columns: prisms with the same centroid xy (the layers of one triangle)
        keys, col_of = np.unique(np.round(cxy, 9), axis=0, return_inverse=True)
        col_of = col_of.reshape(-1)
        col_size = np.bincount(col_of, minlength=keys.shape[0])
        order = np.lexsort((keys[:, 1 - axis], keys[:, axis]))
        cum = np.cumsum(col_size[order])
        total = cum[-1] if cum.size else 0
        strip_of_col = np.empty(keys.shape[0], dtype=np.int64)
        # column k of the sorted order goes to the strip its prism count falls in
        strip_of_col[order] = np.minimum((n_parts * (cum - col_size[order])) // max(total, 1), n_parts - 1)
        self.elem_part = strip_of_col[col_of]
        owner = np.full(self.n_nodes, n_parts, dtype=np.int64)
        for a in range(6):
            np.minimum.at(owner, c[:, a], self.elem_part)
        if np.any(owner == n_parts):
            raise ValueError("a node belongs to no prism")
        self.node_owner = owner
        # node adjacency (nodes sharing a prism), for the solve halo
        rows = np.repeat(c, 6, axis=1).reshape(-1)
        cols = np.tile(c, (1, 6)).reshape(-1)
        adj = np.unique(rows * self.n_nodes + cols)
        self._adj_r, self._adj_c = adj // self.n_nodes, adj % self.n_nodes
        self.conn = c
        self.ranks = [self._rank(r) for r in range(n_parts)]

    def _rank(self, r):
        elems = np.flatnonzero(self.elem_part == r)
        touched = np.unique(self.conn[elems].reshape(-1))
        owned = np.flatnonzero(self.node_owner == r)
        ghosts_asm = touched[self.node_owner[touched] != r]
        nb = self._adj_c[np.isin(self._adj_r, owned)]
        ghosts_spmv = np.unique(nb[self.node_owner[nb] != r])
        return {"elems": elems, "owned": owned, "asm_ghosts": ghosts_asm, "spmv_ghosts": ghosts_spmv,
                "submesh_nodes": touched}

    def submesh(self, t, r):
        """The rank's prisms as a tissue of their own (nodes renumbered in
        ascending global order) and the global ids of its nodes."""
        from .mesh import Tissue

        R = self.ranks[r]
        nodes = R["submesh_nodes"]
        remap = np.full(self.n_nodes, -1, dtype=np.int64)
        remap[nodes] = np.arange(nodes.size)
        e = R["elems"]
        conn = remap[self.conn[e]].astype(np.int32).reshape(-1)
        node3 = (3 * nodes[:, None] + np.arange(3)[None, :]).reshape(-1)
        elem3 = (3 * e[:, None] + np.arange(3)[None, :]).reshape(-1)
        sub = Tissue(pos=np.asarray(t.pos).reshape(-1)[node3], conn=conn,
                     fixed=np.asarray(t.fixed).reshape(-1)[node3], ext_visc=np.asarray(t.ext_visc).reshape(-1)[node3],
                     node_placement=np.asarray(t.node_placement)[nodes], E=np.asarray(t.E)[e],
                     nu=np.asarray(t.nu)[e], eta=np.asarray(t.eta)[e], rates=np.asarray(t.rates).reshape(-1)[elem3],
                     dt=t.dt, n_steps=t.n_steps, name=f"{t.name}-part{r}")
        return sub, nodes


class Comm:
    """Point-to-point exchange and sums over torch.distributed."""

    def __init__(self, dist, device="cpu"):
        import torch

        self.dist, self.torch, self.device = dist, torch, device
        self.rank, self.world = dist.get_rank(), dist.get_world_size()

    def exchange(self, send: dict, recv_sizes: dict) -> dict:
        """Sends send[q] (1-D float64 arrays) to ranks q and receives
        recv_sizes[q] values from each q."""
        torch = self.torch
        reqs, out = [], {}
        for q, n in recv_sizes.items():
            out[q] = torch.empty(int(n), dtype=torch.float64, device=self.device)
            reqs.append(self.dist.irecv(out[q], src=q))
        keep = []
        for q, a in send.items():
            tns = torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64)).to(self.device)
            keep.append(tns)
            reqs.append(self.dist.isend(tns, dst=q))
        for rq in reqs:
            rq.wait()
        return {q: v.cpu().numpy() for q, v in out.items()}

    def exchange_sized(self, send: dict, peers) -> dict:
        """exchange() when the receiver does not know the sizes: the sizes go
        first."""
        sizes = self.exchange({q: np.array([float(np.asarray(send.get(q, [])).size)]) for q in peers},
                              {q: 1 for q in peers})
        return self.exchange({q: send.get(q, np.zeros(0)) for q in peers},
                             {q: int(sizes[q][0]) for q in peers})

    def allreduce(self, a):
        t = self.torch.as_tensor(np.atleast_1d(np.asarray(a, dtype=np.float64))).to(self.device)
        self.dist.all_reduce(t)
        return t.cpu().numpy()


class RankSystem:
    """The owned rows of A = K^T and g on one rank after the assembly halo,
    and the distributed operations of the Krylov solve."""

    def __init__(self, part: StripPartition, rank: int, comm: Comm):
        self.part, self.r, self.comm = part, rank, comm
        R = part.ranks[rank]
        self.owned = R["owned"]
        self.ghosts = R["spmv_ghosts"]
        self.cols = np.concatenate([self.owned, self.ghosts])  # local column order
        self.col_of = np.full(part.n_nodes, -1, dtype=np.int64)
        self.col_of[self.cols] = np.arange(self.cols.size)
        peers = sorted(set(range(part.n_parts)) - {rank})
        self.peers = peers
        # solve halo: who needs which of my owned nodes, whose nodes I need
        self.send_nodes = {q: np.intersect1d(part.ranks[q]["spmv_ghosts"], self.owned) for q in peers}
        self.recv_nodes = {q: self.ghosts[part.node_owner[self.ghosts] == q] for q in peers}

    # -- assembly -------------------------------------------------------------
    def assemble(self, sub_nodes, Ke, Kv, fe, fv, area, vel, dt, ext_visc, fixed):
        """Owned rows of A and g from the rank's element quantities.

        sub_nodes: global ids of the submesh's nodes; Ke, Kv (m, 18, 18) and
        fe, fv (m, 6, 3) of the rank's prisms in submesh numbering (reference
        orientation); area: the submesh nodes' viscosity areas from the rank's
        own prisms (partial at the interface); vel (3 per submesh node); the
        global fixed and ext_visc arrays (3 per node).  Follows the
        reference's assembly (NewtonRaphsonSolver.cpp:273-378 and
        calcutateFixedK :237-255) on the owned rows."""
        part, r = self.part, self.r
        e = part.ranks[r]["elems"]
        conn_g = part.conn[e]                                    # global node ids (m, 6)
        dof = (3 * conn_g[:, :, None] + np.arange(3)[None, None, :]).reshape(len(e), 18)
        Kel = np.asarray(Ke) + np.asarray(Kv)
        # K[dof_a][dof_b] += Kel[a][b]  ->  A[dof_b][dof_a] (A = K^T)
        arow = np.broadcast_to(dof[:, None, :], Kel.shape).reshape(-1)   # A row = K column
        acol = np.broadcast_to(dof[:, :, None], Kel.shape).reshape(-1)
        aval = Kel.reshape(-1)
        gl = np.zeros(3 * part.n_nodes)
        np.add.at(gl, dof.reshape(-1), (np.asarray(fe) + np.asarray(fv)).reshape(-1))
        ar = np.zeros(part.n_nodes)
        ar[sub_nodes] = area
        # the assembly halo: interface rows, g and areas to their owners
        row_owner = part.node_owner[arow // 3]
        mine = row_owner == r
        send, need = {}, {}
        for q in self.peers:
            m = row_owner == q
            gn = part.ranks[r]["asm_ghosts"]
            gn = gn[part.node_owner[gn] == q]
            g3 = (3 * gn[:, None] + np.arange(3)[None, :]).reshape(-1)
            send[q] = np.concatenate([arow[m].astype(np.float64), acol[m].astype(np.float64), aval[m],
                                      gn.astype(np.float64), gl[g3], ar[gn]])
            need[q] = (int(m.sum()), gn.size)
        got = self.comm.exchange_sized(send, self.peers)
        arow_o, acol_o, aval_o = [arow[mine]], [acol[mine]], [aval[mine]]
        g_own = gl.copy()
        ar_own = ar.copy()
        for q in self.peers:
            v = got[q]
            if v.size == 0:
                continue
            # the sender's layout: 3 n entries, then k nodes, 3 k g values, k areas
            k = self._ghost_count_from(q)
            n = (v.size - 5 * k) // 3
            arow_o.append(v[:n].astype(np.int64))
            acol_o.append(v[n:2 * n].astype(np.int64))
            aval_o.append(v[2 * n:3 * n])
            nodes = v[3 * n:3 * n + k].astype(np.int64)
            g3 = (3 * nodes[:, None] + np.arange(3)[None, :]).reshape(-1)
            g_own[g3] += v[3 * n + k:3 * n + 4 * k]
            ar_own[nodes] += v[3 * n + 4 * k:]
        arow_o = np.concatenate(arow_o)
        acol_o = np.concatenate(acol_o)
        aval_o = np.concatenate(aval_o)
        fixed = np.asarray(fixed).reshape(-1).astype(bool)
        ev = np.asarray(ext_visc).reshape(-1)
        own3 = (3 * self.owned[:, None] + np.arange(3)[None, :]).reshape(-1)
        velg = np.zeros(3 * part.n_nodes)
        sub3 = (3 * np.asarray(sub_nodes)[:, None] + np.arange(3)[None, :]).reshape(-1)
        velg[sub3] = vel
        # external viscosity (surface based, NewtonRaphsonSolver.cpp:297-348)
        sv = np.repeat(ar_own[self.owned], 3) * ev[own3]
        arow_o = np.concatenate([arow_o, own3])
        acol_o = np.concatenate([acol_o, own3])
        aval_o = np.concatenate([aval_o, sv / dt])
        g = g_own[own3] - sv * velg[own3]
        # fixed DOFs: row and column zero, diagonal one, g zero
        keep = ~(fixed[arow_o] | fixed[acol_o])
        arow_o, acol_o, aval_o = arow_o[keep], acol_o[keep], aval_o[keep]
        fx = own3[fixed[own3]]
        arow_o = np.concatenate([arow_o, fx])
        acol_o = np.concatenate([acol_o, fx])
        aval_o = np.concatenate([aval_o, np.ones(fx.size)])
        g[fixed[own3]] = 0.0
        # local CSR: rows = owned DOFs, columns = (owned, ghost) DOFs
        import scipy.sparse as sp

        lrow = 3 * np.searchsorted(self.owned, arow_o // 3) + arow_o % 3
        lcol = 3 * self.col_of[acol_o // 3] + acol_o % 3
        if np.any(self.col_of[acol_o // 3] < 0):
            raise RuntimeError("a column outside the rank's owned and ghost nodes")
        self.A = sp.csr_matrix((aval_o, (lrow, lcol)), shape=(3 * self.owned.size, 3 * self.cols.size))
        self.A.sum_duplicates()
        self.g = g
        # block-Jacobi: inverses of the owned 3 x 3 diagonal blocks
        D = np.zeros((self.owned.size, 3, 3))
        Ad = self.A[:, : 3 * self.owned.size].tocoo()
        on = (Ad.row // 3) == (Ad.col // 3)
        D[Ad.row[on] // 3, Ad.row[on] % 3, Ad.col[on] % 3] = Ad.data[on]
        self.Dinv = np.linalg.inv(D)
        return self.A, self.g

    def _ghost_count_from(self, q):
        gn = self.part.ranks[q]["asm_ghosts"]
        return int(np.sum(self.part.node_owner[gn] == self.r))

    # -- solve --------------------------------------------------------------------
    def halo(self, x_owned):
        """x on the owned and ghost nodes (the solve halo)."""
        send = {q: x_owned.reshape(-1, 3)[np.searchsorted(self.owned, n)].reshape(-1)
                for q, n in self.send_nodes.items()}
        got = self.comm.exchange(send, {q: 3 * n.size for q, n in self.recv_nodes.items()})
        xg = np.empty(3 * self.ghosts.size)
        for q, n in self.recv_nodes.items():
            idx = np.searchsorted(self.ghosts, n)
            xg.reshape(-1, 3)[idx] = got[q].reshape(-1, 3)
        return np.concatenate([x_owned, xg])

    def matvec(self, x_owned):
        return self.A @ self.halo(x_owned)

    def dot(self, a, b):
        return float(self.comm.allreduce(np.dot(a, b))[0])

    def precond(self, v):
        return np.einsum("nij,nj->ni", self.Dinv, v.reshape(-1, 3)).reshape(-1)

    def bicgstab(self, rtol=1e-12, max_iter=20000):
        """Block-Jacobi preconditioned BiCGStab on the owned rows: A du = g.
        Returns (du on the owned DOFs, iterations, relative residual)."""
        b = self.g
        x = np.zeros_like(b)
        r = b.copy()
        rhat = r.copy()
        bb = self.dot(b, b)
        if bb == 0.0:
            return x, 0, 0.0
        rho = alpha = omega = 1.0
        v = np.zeros_like(b)
        p = np.zeros_like(b)
        it = 0
        rr = bb
        while it < max_iter:
            rho_new = self.dot(rhat, r)
            if rho_new == 0.0:
                raise RuntimeError("BiCGStab breakdown (rho = 0)")
            beta = (rho_new / rho) * (alpha / omega)
            rho = rho_new
            p = r + beta * (p - omega * v)
            ph = self.precond(p)
            v = self.matvec(ph)
            alpha = rho / self.dot(rhat, v)
            s = r - alpha * v
            sh = self.precond(s)
            tv = self.matvec(sh)
            tt = self.dot(tv, tv)
            omega = self.dot(tv, s) / tt if tt > 0 else 0.0
            x = x + alpha * ph + omega * sh
            r = s - omega * tv
            it += 1
            rr = self.dot(r, r)
            if rr <= rtol * rtol * bb:
                break
            if omega == 0.0:
                raise RuntimeError("BiCGStab breakdown (omega = 0)")
        return x, it, float(np.sqrt(rr / bb))
