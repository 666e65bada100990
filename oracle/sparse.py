"""Sparse-storage mode of the oracle, for meshes whose dense K cannot exist.
TEST INFRASTRUCTURE ONLY (tests, fixture generation, the CPU baseline leg of
bench.py); the product never imports it.

The reference keeps K as a dense 3N x 3N matrix (NewtonRaphsonSolver.cpp:33)
and hands Pardiso the value-filtered CSR of it (constructiaForPardiso,
NewtonRaphsonSolver.cpp:686-707) for a transposed solve (iparm[11] = 1,
:418-683).  At 320,000 prisms that dense K would take 2.94 TB.  This module
keeps everything of the oracle's Newton step (``tf_oracle.c``: growth,
viscosity surfaces, the element loop, the scatter of all Kv then all Ke in
element order into the structural CSR, external viscosity, the fixed-DOF
rows and columns, the 1e-13 drop) and replaces only the storage and the
solver:

* the solve of K^T du = g is the **Pardiso stand-in**: a sparse LU
  factorisation (SciPy SuperLU) of K^T in a geometric nested-dissection
  order of the sheet's node columns, used as the preconditioner of GMRES,
  which runs on the current K^T until the normwise backward error
  |g - K^T du| / (|K| |du| + |g|) (infinity norms) is at most
  ``backward_tol`` (1e-14 by default, ~50 units of roundoff: what a direct
  solve with iterative refinement, iparm[7] = 1, reaches on these
  systems).  A factorisation of an older K that no longer gets there is
  redone; a fresh one must reach ``backward_limit`` (1e-13).  The factorisation is kept across Newton iterations and time
  steps and redone when GMRES needs more than ``refactor_after``
  iterations.  Pardiso itself (closed binary, licence-checked) is not
  available; no number produced here is a Pardiso number.
* the Newton loop restates Simulation::updateStepNR
  (Simulation.cpp:6449-6590) as ``tfo_step`` does: ||du||_2 < 1e-8
  (checkConvergenceViaDeltaU, NewtonRaphsonSolver.cpp:727-740), uk += du
  (:755-761), at most 20 (+1) iterations, continue when capped.
"""
from __future__ import annotations

import time

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as sla

from .oracle import CLOSED, Port


def nested_dissection(xy: np.ndarray, leaf: int = 64, band: float = 2.6) -> np.ndarray:
    """Node order of a geometric nested dissection of a sheet whose nodes lie
    in columns (all layers of one xy position): recursive halving across the
    longer extent, the nodes within ``band`` of the median line forming the
    separator, ordered after both halves.  Nodes of one column stay
    together.  Returns a permutation of ``arange(len(xy))``."""
    out = []

    def rec(ids):
        if ids.size <= leaf:
            out.append(ids)
            return
        p = xy[ids]
        ext = p.max(axis=0) - p.min(axis=0)
        ax = int(ext[1] > ext[0])
        med = np.median(p[:, ax])
        lo = p[:, ax] < med - band
        hi = p[:, ax] > med + band
        if not lo.any() or not hi.any():
            out.append(ids)
            return
        rec(ids[lo])
        rec(ids[hi])
        out.append(ids[~(lo | hi)])

    rec(np.arange(xy.shape[0]))
    return np.concatenate(out)


class TransposedSolve:
    """K^T du = g to a normwise backward error ``backward_tol`` (the Pardiso
    stand-in)."""

    def __init__(self, node_xy: np.ndarray, rtol: float = 1e-14, refactor_after: int = 30,
                 band: float = 2.6, backward_tol: float = 1e-14, backward_limit: float = 1e-13):
        nodes = nested_dissection(np.asarray(node_xy, dtype=np.float64), band=band)
        self.perm = (3 * nodes[:, None] + np.arange(3)[None, :]).reshape(-1)
        self.rtol = rtol
        self.backward_tol = backward_tol
        self.backward_limit = backward_limit
        self.refactor_after = refactor_after
        self.lu = None
        self.stats = {"factorisations": 0, "factor_s": 0.0, "solve_s": 0.0, "gmres_iters": []}

    def _factor(self, A):
        t0 = time.time()
        self.lu = sla.splu(A, permc_spec="NATURAL", diag_pivot_thresh=0.1,
                           options=dict(SymmetricMode=True))
        self.stats["factorisations"] += 1
        self.stats["factor_s"] += time.time() - t0

    def solve(self, ia, ja, a, g):
        """du with K^T du = g, K given as the reference's CSR (ia, ja, a)."""
        n = g.size
        # CSC arrays of K are the CSR arrays of K^T
        A = sp.csc_matrix((a, ja, ia), shape=(n, n))[self.perm][:, self.perm].tocsc()
        b = g[self.perm]
        if not np.any(b):
            return np.zeros(n)
        anorm = float(np.abs(A).sum(axis=1).max())
        t0 = time.time()
        for attempt in range(2):
            fresh = self.lu is None
            if fresh:
                self._factor(A)
            lu = self.lu
            M = sla.LinearOperator(A.shape, matvec=lambda v: lu.solve(np.asarray(v, dtype=np.float64)))
            count = [0]

            def cb(_):
                count[0] += 1

            x, info = sla.gmres(A, b, M=M, rtol=self.rtol, atol=0.0, restart=100, maxiter=1,
                                callback=cb, callback_type="pr_norm")
            # normwise backward error |b - A x| / (|A| |x| + |b|), infinity norms: what a
            # direct solve with refinement guarantees (near unit roundoff) and what stays
            # meaningful when b is small against the terms A x cancels (late Newton iterations)
            r = b - A @ x
            res = float(np.abs(r).max()) / (anorm * float(np.abs(x).max()) + float(np.abs(b).max()))
            if res <= self.backward_tol or fresh:
                break
            self.lu = None  # the factorisation of an older K no longer serves: redo it
        if count[0] > self.refactor_after:
            self.lu = None  # converged, but slowly: factorise the next system afresh
        self.stats["gmres_iters"].append(count[0])
        self.stats["solve_s"] += time.time() - t0
        self.stats["backward_error"] = max(self.stats.get("backward_error", 0.0), res)
        if not res <= self.backward_limit:
            raise RuntimeError(f"Pardiso stand-in did not converge: backward error {res:.3e}")
        du = np.empty(n)
        du[self.perm] = x
        return du


def newton_step(port: Port, solver: TransposedSolve, dt: float, rates=None, mode: int = CLOSED,
                max_iter: int = 20, tol: float = 1e-8):
    """One time step of the oracle with sparse storage: growth and viscosity
    surfaces of the step's start (runOneStep, Simulation.cpp:5906-5915), then
    the Newton loop of updateStepNR (Simulation.cpp:6449-6590).  Returns the
    iteration count, the ||du|| history and whether the loop was capped."""
    if rates is not None:
        port.grow(dt, rates)
    port.update_viscosity_surfaces()
    un = port.positions()
    uk = un.copy()
    hist = []
    k, converged, capped = 0, False, False
    while not converged:
        port.assemble(uk, un, dt, mode)
        ia, ja, a = port.export_filtered(1e-13)
        g = port.rhs()
        du = solver.solve(ia, ja, a, g)
        d = float(np.sqrt(np.sum(du * du)))
        hist.append(d)
        converged = not (d > tol)
        uk = uk + du
        k += 1
        if not converged and k > max_iter:
            capped = converged = True
    port.set_positions(uk)
    return {"iters": k, "dunorm": np.array(hist), "capped": capped}
