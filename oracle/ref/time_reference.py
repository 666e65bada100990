"""Times the reference's own compiled hot path (oracle/_ref/libtfref.so: the
reference's ShapeBase / Prism / Node / NewtonRaphsonSolver sources compiled
unmodified, GSL and Pardiso replaced by the project's stand-ins) on this
host's cores, phase by phase, next to the oracle port.  TEST / MEASUREMENT
INFRASTRUCTURE: it runs only where the reference checkout is present.

    OMP_NUM_THREADS=8 python oracle/ref/time_reference.py

Phases of one Newton iteration of the 1,600-prism configuration (config 1):
  * the element loop (NewtonRaphsonSolver::calculateForcesAndJacobianMatrixNR,
    NewtonRaphsonSolver.cpp:257-271, OpenMP over prisms);
  * everything else up to the solve: the serial scatter into the dense K and
    g, external viscosity, fixed DOFs and the dense -> CSR scan
    (NewtonRaphsonSolver.cpp:273-348, :237-255, :686-724);
  * the transposed solve (the Pardiso stand-in: banded LU);
  * whole implicit steps (growth, viscosity surfaces, the Newton loop).
The element loop of the 320,000-prism configuration's element type (internal
viscosity 100, log-normal E) is timed on its 12,800-prism sheet (the
reference keeps K dense, 3N x 3N: 5 GB here, 2.94 TB at 320,000 prisms; the
element loop's cost per prism does not depend on the mesh size).
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import LITERAL, Port, Ref  # noqa: E402
from tissuefolding_paperversion_gb300 import mesh  # noqa: E402


def best(f, reps=3):
    out = []
    for _ in range(reps):
        t0 = time.perf_counter()
        f()
        out.append(time.perf_counter() - t0)
    return min(out)


def main():
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    Port.set_threads(threads)
    rows = {}
    # config 1
    t = mesh.config_small(seed=0)
    r = Ref(t)
    p = Port(t)
    uk, un = mesh.perturbed_state(t, seed=1, amp=0.05)
    r.update_viscosity_surfaces()
    p.update_viscosity_surfaces()
    elem = best(lambda: r.element_eval(uk, un, t.dt))
    asm = best(lambda: r.assemble(uk, un, t.dt))
    elem_port = best(lambda: p.element_eval(uk, un, t.dt, LITERAL))
    rows["config1_element_loop_ms"] = elem * 1e3
    rows["config1_prisms_per_s_reference"] = t.n_elems / elem
    rows["config1_prisms_per_s_port"] = t.n_elems / elem_port
    rows["config1_assembly_to_csr_ms"] = asm * 1e3
    rows["config1_scatter_bc_csr_ms"] = (asm - elem) * 1e3
    r.close()
    r = Ref(t)
    r.step(t.dt, t.rates)  # warm-up
    steps, its = [], []
    for _ in range(3):
        t0 = time.perf_counter()
        out = r.step(t.dt, t.rates)
        steps.append(time.perf_counter() - t0)
        its.append(out["iters"])
    step = float(np.median(steps))
    rows["config1_step_ms"] = step * 1e3
    rows["config1_newton_iters_per_step"] = float(np.mean(its))
    rows["config1_solve_ms_per_iteration"] = (step / np.mean(its) - asm) * 1e3
    r.close()
    # config 2 element type, on its 12,800-prism sheet
    t2 = mesh.config_large(seed=0, cells=40)
    r2 = Ref(t2)
    p2 = Port(t2)
    uk2, un2 = mesh.perturbed_state(t2, seed=1, amp=0.05)
    e2 = best(lambda: r2.element_eval(uk2, un2, t2.dt), reps=2)
    e2p = best(lambda: p2.element_eval(uk2, un2, t2.dt, LITERAL), reps=2)
    rows["config2_element_prisms_per_s_reference"] = t2.n_elems / e2
    rows["config2_element_prisms_per_s_port"] = t2.n_elems / e2p
    rows["config2_element_loop_ms_per_320k_prisms"] = 320000 / (t2.n_elems / e2) * 1e3
    rows["threads"] = threads
    rows["host"] = os.uname().machine
    print(json.dumps(rows, indent=1))


if __name__ == "__main__":
    main()
