"""Generates tests/golden/steps_large_320k.npz: 20 implicit time steps of the
320,000-prism sheet (200 x 200 cells, 4 layers, E log-normal, internal
viscosity 100 Pa s, Gaussian growth bump, dt = 60 s; seed 0) computed by the
oracle in sparse-storage mode.

    python tests/golden/make_large_steps.py [--cells 200] [--steps 20] [--threads 8]

The element loop, scatter order, boundary conditions and Newton loop are the
oracle's restatement of the reference (``oracle/tf_oracle.c``, pinned bit for
bit to the reference's own sources by tests/test_oracle.py; the tangent in its
closed form, within 1e-12 of the literal 3^6 contraction).  The reference's
dense K cannot exist at this size (2.94 TB), so the storage is the
reference's value-filtered CSR and the solver is the Pardiso stand-in of
``oracle/sparse.py`` (sparse LU as the preconditioner of GMRES, run to a
normwise backward error of 1e-14).

The fixture keeps what a GPU run can be compared with at any size: the Newton
iteration count and ||du|| of every iteration of every step, per-step
checksums of all positions, and the positions of 2,048 seeded nodes after
every step.  It takes about an hour on 8 cores.
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import sparse  # noqa: E402
from oracle.oracle import CLOSED, Port  # noqa: E402
from tissuefolding_paperversion_gb300 import mesh  # noqa: E402

N_SAMPLE = 2048


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--cells", type=int, default=200)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--out", default=None)
    args = ap.parse_args()
    t = mesh.config_large(seed=0, cells=args.cells)
    out = args.out or os.path.join(HERE, f"steps_large_{t.n_elems // 1000}k.npz")
    Port.set_threads(args.threads)
    port = Port(t)
    solver = sparse.TransposedSolve(t.pos.reshape(-1, 3)[:, :2])
    sample = np.sort(np.random.default_rng(12345).choice(t.n_nodes, size=min(N_SAMPLE, t.n_nodes),
                                                         replace=False)).astype(np.int32)
    pos0 = t.pos.reshape(-1, 3).copy()
    iters, dun, samp, csum, dnorm, dmax, step_s = [], [], [], [], [], [], []
    t_all = time.time()
    for s in range(args.steps):
        t0 = time.time()
        r = sparse.newton_step(port, solver, t.dt, t.rates, mode=CLOSED)
        step_s.append(time.time() - t0)
        p = port.positions().reshape(-1, 3)
        d = np.zeros(21)
        d[: len(r["dunorm"])] = r["dunorm"][:21]
        iters.append(r["iters"])
        dun.append(d)
        samp.append(p[sample].copy())
        csum.append(p.sum(axis=0))
        disp = p - pos0
        dnorm.append(np.linalg.norm(disp))
        dmax.append(np.abs(disp).max())
        print(f"step {s}: {r['iters']} Newton iterations, |du| {r['dunorm']}, {step_s[-1]:.1f} s, "
              f"GMRES {solver.stats['gmres_iters'][-r['iters']:]}, factorisations {solver.stats['factorisations']}",
              flush=True)
    np.savez_compressed(
        out, seed=0, cells=args.cells, dt=t.dt, n_prisms=t.n_elems, n_nodes=t.n_nodes,
        iters=np.array(iters, dtype=np.int32), dunorm=np.array(dun), sample_nodes=sample,
        sample_positions=np.array(samp), position_sums=np.array(csum), disp_norm=np.array(dnorm),
        disp_max=np.array(dmax), step_seconds=np.array(step_s), threads=args.threads,
        factorisations=solver.stats["factorisations"], factor_seconds=solver.stats["factor_s"],
        gmres_iters=np.array(solver.stats["gmres_iters"], dtype=np.int32),
        backward_error=solver.stats.get("backward_error", 0.0),
        note="oracle sparse mode: tf_oracle.c closed-form tangent, reference scatter order and CSR filter, "
             "Pardiso stand-in = SuperLU (nested dissection) preconditioned GMRES to backward error 1e-14")
    print(f"wrote {out} in {time.time() - t_all:.0f} s", flush=True)


if __name__ == "__main__":
    main()
