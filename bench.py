"""Benchmark of the GB300 implicit prism step.

Workload: the 320k-prism sheet (200 x 200 cell grid, 4 layers, 202005 nodes,
606015 DOF, E log-normal, internal viscosity 100 Pa s, Gaussian growth bump),
one implicit time step of 60 s per bench step.

Reported (one JSON line on rank 0):
  value        prism K+f assemblies/s: prisms x assemblies / device time of
               the assemblies, measured inside the timed Newton steps
  ms_per_step  Newton-step device time (the whole updateStepNR: growth,
               viscosity surfaces, every assembly and linear solve)
  e2e          the same metric through the C ABI from host buffers: per step
               tf_set_state (H2D of uk, un), tf_assemble, tf_get_residual (D2H)
  roofline     element kernel: algorithmic bytes / kernel time vs measured HBM
  fp64         element kernel: FP64 flops / kernel time vs GB300's FP64 peak
               (the kernel's binding roofline)
  cpu_baseline the reference's algorithm (oracle port, literal 3^6 tangent),
               all host threads, on a bounded sample of prisms
  e2e_newton_step  the whole Newton step through the C ABI with host
               positions in and out (tf_set_positions, tf_newton_step,
               tf_get_positions), wall clock
  config_small the 1,600-prism configuration: GPU Newton step against the
               CPU port's whole step (banded-LU stand-in for Pardiso)
  batch        256 seeded instances (1k-50k prisms) advanced in one handle
               against the plain GPU step looped over a stratified subset
  adjoint      gradient through 50 steps of the 320k-prism sheet
               (checkpoints every 10): backward / forward cost, and the
               gradient against central differences along seeded directions;
               fd_32_directions: 32 directions, 4-point differences, on a
               3,200-prism sheet of the same kind (50 steps)
(`--quick` leaves the last three out.)

`--impl reference` times the CPU implementation alone on the same metric:
each timed step is one bounded sample of the assembly; the full-assembly
time it implies is reported under a key that says it is a projection.
Inputs (~1.3 GB of device data per assembly) exceed the 129 MB L2, so no
flush is needed between timed iterations.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

MEASURED = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM = 6800.0


def peaks():
    try:
        with open(MEASURED) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM, "fallback"


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, index=0):
        self.p = None
        self.path = os.path.join("/tmp", f"tf_clocks_{os.getpid()}.csv")
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def algorithmic_bytes(nn, ne, nnz):
    """Minimal unique traffic of one K+f assembly: per prism 6 int32 node ids,
    18 FP64 reference coordinates, 9 FP64 InvFg, 3 FP64 material values and 36
    int32 slot offsets (408 B); per node uk and un (48 B) and g (24 B); K
    written once (8 B per nonzero)."""
    return 408 * ne + 48 * nn + 24 * nn + 8 * nnz


# Instruction mix of one element-kernel launch, counted with ncu on the
# 135,200-prism sheet with internal viscosity (per prism): FP64 flops
# (2 x DFMA + DADD + DMUL thread instructions; phase A and the joins) and
# FP32 thread instructions (FADD + FFMA + FMUL; the double-float block sums),
# with the FP64 pipe's busy fraction ncu reported.  The elastic-only counts
# apply when every eta is 0 (not captured).
FP64_FLOPS_PER_PRISM = {"viscous": 4644, "elastic": None}
FP32_INST_PER_PRISM = {"viscous": 136492, "elastic": None}
FP64_PIPE_PCT_NCU = {"viscous": 44.1, "elastic": None}
# DRAM bytes (read + write) per prism of one element-kernel launch, from the
# same ncu capture (333.1 MB at 135,200 prisms); the kernel's traffic grows
# with the number of prisms, so a full launch is scaled from it.
DRAM_BYTES_PER_PRISM = {"viscous": 333.1e6 / 135200, "elastic": None}
FP64_PEAK_TFLOPS = 304 * 2 * 2.07e9 / 1e12


def cpu_sample(t, seconds_target=15.0, literal=True):
    """The reference's algorithm on the host: element loop + serial scatter on
    a bounded sample of prisms; returns (prisms/s, sample, threads)."""
    from oracle.oracle import CLOSED, LITERAL, Port

    p = Port(t)
    uk, un = t.pos + 0.01, t.pos
    mode = LITERAL if literal else CLOSED
    n = 256
    p.assemble_sample(uk, un, t.dt, 64, mode)   # warm-up
    t0 = time.perf_counter()
    p.assemble_sample(uk, un, t.dt, n, mode)
    dt = time.perf_counter() - t0
    rate = n / dt
    n = int(min(t.n_elems, max(256, rate * seconds_target)))
    t0 = time.perf_counter()
    p.assemble_sample(uk, un, t.dt, n, mode)
    dt = time.perf_counter() - t0
    p.close()
    return n / dt, n, dt, Port.threads()


def cpu_newton_small(steps=2):
    """The reference's own CPU-runnable case (1,600 prisms, 3,969 DOF): whole
    implicit steps of the oracle port (literal 3^6 tangent, the reference's
    scatter and CSR filter, banded-LU stand-in for Pardiso), all host
    threads.  Returns (ms per step, Newton iterations per step, threads)."""
    from oracle.oracle import LITERAL, Port
    from tissuefolding_paperversion_gb300 import mesh

    t = mesh.config_small(seed=0)
    p = Port(t)
    p.step(t.dt, t.rates, LITERAL)   # warm-up
    its = []
    t0 = time.perf_counter()
    for _ in range(steps):
        its.append(p.step(t.dt, t.rates, LITERAL)["iters"])
    ms = (time.perf_counter() - t0) / steps * 1e3
    p.close()
    return ms, float(np.mean(its)), Port.threads()


def recorded_cpu_newton_large():
    """The CPU Newton step of the 320,000-prism sheet as recorded when its
    20-step oracle run was made (oracle port, closed-form tangent, sparse
    storage, SuperLU-preconditioned GMRES as the Pardiso stand-in)."""
    f = os.path.join(ROOT, "tests", "golden", "steps_large_320k.npz")
    if not os.path.exists(f):
        return None
    d = np.load(f)
    return {"ms_per_step_median": float(np.median(d["step_seconds"])) * 1e3,
            "ms_first_step_with_factorisation": float(d["step_seconds"][0]) * 1e3,
            "newton_iters_per_step": float(np.mean(d["iters"])), "threads": int(d["threads"]),
            "how": "recorded when tests/golden/steps_large_320k.npz was made (8-core x86 host), not in this run"}


def small_config_measure(args):
    """GPU vs CPU Newton step on the 1,600-prism configuration."""
    from tissuefolding_paperversion_gb300 import api, mesh

    t = mesh.config_small(seed=0)
    with api.Solver(t) as s:
        s.set_growth_rates(t.rates)
        for _ in range(3):
            s.newton_step(t.dt)
        outs = [s.newton_step(t.dt) for _ in range(10)]
    gpu_ms = float(np.mean([o["ms_total"] for o in outs]))
    out = {"workload": t.name, "prisms": t.n_elems, "gpu_ms_per_step": gpu_ms,
           "gpu_krylov_iters_per_step": float(np.mean([o["krylov_total"] for o in outs]))}
    if not args.no_cpu_baseline:
        ms, its, th = cpu_newton_small()
        out.update({"cpu_ms_per_step": ms, "cpu_cores": th, "cpu_kind": "port",
                    "cpu_newton_iters_per_step": its, "cpu_over_gpu": ms / gpu_ms})
    return out


def run_reference(args, t):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle.oracle import Port

    Port.set_threads(os.cpu_count() or 1)
    rates = []
    for _ in range(args.warmup):
        cpu_sample(t, seconds_target=1.0)
    samples, secs = [], []
    w0 = time.perf_counter()
    for _ in range(args.steps):
        r, n, dt, th = cpu_sample(t, seconds_target=args.ref_seconds)
        rates.append(r)
        samples.append(n)
        secs.append(dt)
    wall = time.perf_counter() - w0
    value = statistics.median(rates)
    ms_small, its_small, th_small = cpu_newton_small()
    line = {
        "impl": "reference", "metric": "prism K+f assemblies/s", "value": value, "unit": "prisms/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": t.name, "prisms": t.n_elems, "nodes": t.n_nodes, "dof": 3 * t.n_nodes,
                   "l2": "inputs larger than L2"},
        # each timed step is one bounded sample of the assembly (its prisms below)
        "ms_per_step": wall / args.steps * 1e3,
        "prisms_per_step": int(statistics.median(samples)),
        "projected_ms_per_full_assembly": t.n_elems / value * 1e3,
        "projection": "prisms of the workload / measured prisms/s; not timed as one piece",
        "cpu_baseline": {"value": value, "unit": "prisms/s", "cores": Port.threads(), "kind": "port",
                         "sample": f"element loop (literal 3^6 tangent, the reference's algorithm) + serial "
                                   f"scatter over the first {samples[-1]} of {t.n_elems} prisms per step"},
        "e2e": {"value": value, "unit": "prisms/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "newton_step_cpu": {
            "config_small": {"ms_per_step": ms_small, "newton_iters_per_step": its_small, "cores": th_small,
                             "prisms": 1600,
                             "how": "whole implicit steps of the port (literal tangent, banded-LU stand-in for "
                                    "Pardiso), measured in this run"},
            "config_large": recorded_cpu_newton_large()},
    }
    print(json.dumps(line))


def run_gpu(args, t):
    from tissuefolding_paperversion_gb300 import api

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811

        dist.init_process_group("gloo")
    s = api.Solver(t, device=local if world > 1 else 0, precond=args.precond, host_loops=args.host_loops,
                   multigrid_reuse_steps=args.mg_reuse)
    s.set_growth_rates(t.rates)
    nn, ne, nnzb = s.sizes()
    mg_nodes, _ = s.multigrid_info()
    mg_blocks = s.multigrid_blocks() if mg_nodes else None

    def barrier():
        if dist is not None:
            dist.barrier()

    wstats = [s.newton_step(t.dt) for _ in range(args.warmup)]
    barrier()
    l0 = s.launch_count()
    clocks = Clocks(local)
    w0 = time.perf_counter()
    stats = [s.newton_step(t.dt) for _ in range(args.steps)]
    wall = time.perf_counter() - w0
    clk = clocks.stop()
    launches = s.launch_count() - l0
    ms_steps = [x["ms_total"] for x in stats]
    ms_asm = sum(x["ms_assemble"] for x in stats)
    n_asm = sum(x["iters"] for x in stats)
    step_ms = sum(ms_steps) / len(ms_steps)
    asm_rate = ne * n_asm / (ms_asm / 1e3)
    if dist is not None:
        import torch

        v = torch.tensor([step_ms, ms_asm / n_asm], dtype=torch.float64)
        dist.all_reduce(v, op=dist.ReduceOp.MAX)
        step_ms, per_asm = float(v[0]), float(v[1])
        asm_rate = ne * world / (per_asm / 1e3)

    tiles = s.tiles()
    # element-kernel roofline (back-to-back assemblies at the converged state)
    per_asm_ms, elem_ms = s.time_assembly(max(3, args.steps))
    ia, ja, a = s.export_csr(0.0)
    nnz = int(ia[-1])
    alg = algorithmic_bytes(nn, ne, nnz)
    hbm, how = peaks()
    achieved = alg / (elem_ms / 1e3) / 1e9
    # the kernel's binding roofline: FP64 issue (see profiles/)
    kind = "viscous" if np.any(t.eta != 0) else "elastic"
    fpp = FP64_FLOPS_PER_PRISM[kind]
    traffic = DRAM_BYTES_PER_PRISM[kind] * ne if DRAM_BYTES_PER_PRISM[kind] else None
    fp64 = None
    if fpp:
        tf = fpp * ne / (elem_ms / 1e3) / 1e12
        fp64 = {"kernel": "k_element", "achieved": tf, "peak": FP64_PEAK_TFLOPS, "unit": "TFLOP/s",
                "frac": tf / FP64_PEAK_TFLOPS, "flops_per_prism": fpp,
                "peak_source": "ncu peak_sustained DFMA rate x max SM clock",
                "fp64_pipe_pct_ncu": FP64_PIPE_PCT_NCU[kind],
                "fp32_inst_per_prism": FP32_INST_PER_PRISM[kind],
                "note": "phase A and the forces in FP64; the tangent's block sums in double-float on the FP32 pipe"}

    # e2e through the C ABI with host buffers
    uk = s.positions()
    un = uk - 1e-3
    for _ in range(2):
        s.set_state(uk, un, t.dt)
        s.assemble()
        s.residual()
    e0 = time.perf_counter()
    for _ in range(args.steps):
        s.set_state(uk, un, t.dt)
        s.assemble()
        g = s.residual()
    e2e_s = (time.perf_counter() - e0) / args.steps
    # the whole Newton step through the C ABI as the reference's caller uses it
    # (tf_set_positions from host memory, tf_newton_step, tf_get_positions back)
    host = s.positions()
    for _ in range(2):
        s.set_positions(host)
        s.newton_step(t.dt)
        host = s.positions()
    e0 = time.perf_counter()
    dev_ms = 0.0
    for _ in range(args.steps):
        s.set_positions(host)
        dev_ms += s.newton_step(t.dt)["ms_total"]
        host = s.positions()
    e2e_step_ms = (time.perf_counter() - e0) / args.steps * 1e3
    s.close()
    e2e_step = {"ms_per_step": e2e_step_ms, "device_ms_per_step": dev_ms / args.steps,
                "calls": "tf_set_positions (H2D), tf_newton_step, tf_get_positions (D2H)",
                "h2d_bytes_per_step": 8 * 3 * nn, "d2h_bytes_per_step": 8 * 3 * nn}
    small = None if args.quick else small_config_measure(args)
    batch = None
    if not args.quick and world == 1:
        from tissuefolding_paperversion_gb300 import mesh

        ts = [mesh.config_batch_instance(k) for k in range(args.instances)]
        batch = batch_measure(ts, 3, 1, loop_every=8)
        batch["instances"] = len(ts)
        batch["prisms"] = int(sum(x.n_elems for x in ts))
    adjoint = None
    if not args.quick and world == 1:
        adjoint = adjoint_measure(t, args.adj_steps, args.adj_every, args.adj_fd_default)
        adjoint["fd_32_directions"] = adjoint_fd_sheet()
    # the read and copy bandwidth this GPU gives kernels of the library (the
    # denominators of the solve's read-bound kernels)
    hbm_probe = api.measure_bandwidth(local if world > 1 else 0)
    if rank != 0:
        return
    line = {
        "metric": "prism K+f assemblies/s", "value": asm_rate, "unit": "prisms/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": t.name, "prisms": ne, "nodes": nn, "dof": 3 * nn, "block_nonzeros": nnzb,
                   "dt_s": t.dt, "l2": "inputs larger than L2 (no flush)", "parallelism": "replicas" if world > 1 else "single"},
        "newton": {"ms_per_step": step_ms, "assemblies_per_step": n_asm / len(stats),
                   "preconditioner": (("plain-aggregation" if args.precond == 3 else "smoothed-aggregation")
                                      + " multigrid " + "/".join(map(str, mg_nodes))) if mg_nodes else "block-Jacobi",
                   "multigrid_blocks": mg_blocks[0] if mg_blocks else None,
                   "autotuned": tiles,
                   "multigrid_reuse_steps": args.mg_reuse if args.mg_reuse else 4,
                   "krylov_iters_per_step": sum(x["krylov_total"] for x in stats) / len(stats),
                   "krylov_iters_by_step": [int(x["krylov_total"]) for x in stats],
                   "newton_iters_by_step": [int(x["iters"]) for x in stats],
                   "device_loop_iters_by_step": [int(x.get("device_iters", 0)) for x in stats],
                   "device_loop_handback_by_step": [int(x.get("device_handback", 0)) for x in stats],
                   "ms_by_step": [round(float(x["ms_total"]), 3) for x in stats],
                   "ms_assembly": ms_asm / n_asm, "wall_s": wall,
                   "warmup_steps": {"krylov_iters_by_step": [int(x["krylov_total"]) for x in wstats],
                                    "newton_iters_by_step": [int(x["iters"]) for x in wstats],
                                    "ms_by_step": [round(float(x["ms_total"]), 3) for x in wstats]}},
        "e2e": {"value": ne / e2e_s, "unit": "prisms/s", "h2d_bytes_per_step": 2 * 8 * 3 * nn,
                "d2h_bytes_per_step": 8 * 3 * nn},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic, "peak_source": how, "kernel": "k_element", "ms_per_launch": elem_ms,
                     "algorithmic_bytes": alg,
                     "traffic_source": "ncu dram bytes per prism at 135,200 prisms x prisms" if traffic else None},
        "fp64": fp64,
        "gpu_launches": launches,
        "clocks": clk,
        "e2e_newton_step": e2e_step,
        "hbm_probe": hbm_probe,
    }
    if small is not None:
        line["config_small"] = small
    if batch is not None:
        line["batch"] = batch
    if adjoint is not None:
        line["adjoint"] = adjoint
    if not args.no_cpu_baseline:
        r, n, dt, th = cpu_sample(t, seconds_target=max(args.ref_seconds, 12.0))
        line["cpu_baseline"] = {"value": r, "unit": "prisms/s", "cores": th, "kind": "port",
                                "sample": f"element loop (literal 3^6 tangent) + serial scatter over "
                                          f"{n} of {ne} prisms, {dt:.1f} s"}
    print(json.dumps(line))


def run_assembly_only(args, t):
    """Back-to-back assemblies at a grown state (for kernel profiling)."""
    from tissuefolding_paperversion_gb300 import api

    s = api.Solver(t)
    s.set_growth_rates(t.rates)
    s.begin_step(t.dt)
    uk = t.pos + 1e-3 * np.sin(t.pos)
    s.set_state(uk, t.pos, t.dt)
    s.time_assembly(args.warmup)
    per_asm, elem = s.time_assembly(args.steps)
    print(json.dumps({"mode": "assembly", "workload": t.name, "prisms": t.n_elems, "ms_per_assembly": per_asm,
                      "ms_element_kernel": elem, "prisms_per_s": t.n_elems / (per_asm / 1e3)}))
    s.close()


def batch_measure(ts, steps, warmup, loop_every=1, dev=0, dist=None):
    """The batched sweep on this rank's instances `ts`: one handle advancing
    all of them (per-instance Newton counts and convergence masks, CUDA-graph
    chunks, autotuned elements per CTA) against the plain GPU step looped
    over them, one handle each.  With loop_every = k > 1 the loop is timed
    over every k-th instance in size order (a stratified subset) and its
    rate stands for the whole loop.  Rates are instance time steps
    (implicit solves) per second of wall clock; under torch.distributed the
    times are the max over ranks."""
    from tissuefolding_paperversion_gb300 import api, shard

    def slowest(x):
        return shard.max_over_ranks(dist, x) if dist is not None else x

    b = api.Batch(ts, device=dev)
    b.set_growth_rates()
    for _ in range(warmup):
        b.step(ts[0].dt)
    if dist is not None:
        dist.barrier()
    l0 = b.launch_count()
    w0 = time.perf_counter()
    outs = [b.step(ts[0].dt) for _ in range(steps)]
    wall_b = slowest(time.perf_counter() - w0)
    launches = b.launch_count() - l0
    ms_b = slowest(sum(o["ms_total"] for o in outs))
    ept = b.elements_per_cta()
    b.close()
    order = np.argsort([t.n_elems for t in ts], kind="stable")
    loop_ids = [int(i) for i in order[::loop_every]]
    solvers = []
    for i in loop_ids:
        s = api.Solver(ts[i], device=dev)
        s.set_growth_rates(ts[i].rates)
        solvers.append((s, ts[i]))
    for s, t in solvers:
        for _ in range(max(1, warmup)):
            s.newton_step(t.dt)
    loop_steps = max(1, min(steps, 2))
    if dist is not None:
        dist.barrier()
    w0 = time.perf_counter()
    ms_l = 0.0
    for _ in range(loop_steps):
        for s, t in solvers:
            ms_l += s.newton_step(t.dt)["ms_total"]
    wall_l = slowest(time.perf_counter() - w0)
    ms_l = slowest(ms_l)
    for s, _ in solvers:
        s.close()
    rate_b = len(ts) * steps / wall_b
    rate_l = len(loop_ids) * loop_steps / wall_l
    return {"batched": {"value": rate_b, "unit": "instance steps/s", "steps": steps,
                        "ms_per_step": wall_b / steps * 1e3, "device_ms_per_step": ms_b / steps,
                        "newton_iters_max": int(max(o["iters"].max() for o in outs)),
                        "elements_per_cta": ept, "gpu_launches": launches},
            "looped_plain": {"value": rate_l, "unit": "instance steps/s", "steps": loop_steps,
                             "instances_timed": len(loop_ids),
                             "subset": "all instances" if loop_every == 1 else
                             f"every {loop_every}th instance in size order ({len(loop_ids)} of {len(ts)}); "
                             "its rate stands for the whole loop",
                             "device_ms_per_instance_step": ms_l / (loop_steps * len(loop_ids))},
            "speedup_vs_looped": rate_b / rate_l}


def run_batch(args):
    """Batched sweep: 256 tissues of 1k-50k prisms in one handle vs the plain
    GPU step looped over the instances (one handle each).  Metric: instance
    time steps (implicit solves) per second.  Under torchrun the instances are
    sharded over the ranks (balanced by prism count, no exchange; timings are
    the max over ranks), so the total work is fixed: strong scaling."""
    from tissuefolding_paperversion_gb300 import mesh, shard

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811

        dist.init_process_group("gloo")
    n = args.instances
    ts_all = [mesh.config_batch_instance(s) for s in range(n)]
    mine = shard.shard_instances([t.n_elems for t in ts_all], world)[rank]
    ts = [ts_all[i] for i in mine]
    prisms = sum(t.n_elems for t in ts_all)
    r = batch_measure(ts, args.steps, args.warmup, 1, local if world > 1 else 0, dist)
    if rank != 0:
        return
    rate_b = r["batched"]["value"] * (n / len(ts))
    print(json.dumps({
        "metric": "batched implicit solves/s", "value": rate_b, "unit": "instance steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["batched"]["ms_per_step"],
        "higher_is_better": True, "scaling": "strong", "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"batch-{n}", "instances": n, "prisms": prisms,
                   "elements_per_cta": r["batched"]["elements_per_cta"],
                   "parallelism": f"instances sharded over {world} ranks" if world > 1 else "single"},
        "looped_plain": r["looped_plain"],
        "speedup_vs_looped": r["speedup_vs_looped"],
        "batched_device_ms_per_step": r["batched"]["device_ms_per_step"],
        "newton_iters_max": r["batched"]["newton_iters_max"],
        "gpu_launches": r["batched"]["gpu_launches"],
    }))


def adjoint_measure(t, n, every, fd_dirs, seed=1234, fd_h6=0, fd_order4=False):
    """Adjoint of n implicit steps: loss = squared distance of the final
    apical surface to z = 5 exp(-r^2 / (2 40^2)) um (r from the sheet
    centre), gradient with respect to the per-element growth rates and log E;
    states saved every `every` steps and recomputed in between.  Forward and
    backward are timed (device-synchronised wall clock) at the default
    tolerances.  With fd_dirs > 0 the gradient of a run with every solve
    tight (Newton |du| <= 1e-11, Krylov 1e-13) is checked against central
    differences of that run along fd_dirs seeded directions, alternating
    growth rates (h = 1e-3 of the largest rate) and log E (h = 1e-4).  These
    steps balance the difference's truncation against the FP64 rounding of
    the loss (~1.6e7 on the 320k-prism sheet, rounded to ~1e-9 per term over
    40,401 apical nodes): at h = 1e-6 the central difference itself is
    uncertain by ~2e-4 of the derivative."""
    from tissuefolding_paperversion_gb300 import api

    xy = t.pos.reshape(-1, 3)[:, :2]
    c = 0.5 * (xy.min(axis=0) + xy.max(axis=0))
    params = np.array([c[0], c[1], 5.0, 40.0])
    rate = t.rates.reshape(-1, 3)[:, 0].copy()
    logE = np.log(t.E)
    s = api.Solver(t)
    # warm-up: one short forward/backward (graphs, autotuner)
    s.set_positions(t.pos)
    _, sv = s.adjoint_forward(rate, logE, 1, t.dt, 1, params)
    s.adjoint_backward(sv)
    sv.free()
    s.set_positions(t.pos)
    l0 = s.launch_count()
    w0 = time.perf_counter()
    loss, sv = s.adjoint_forward(rate, logE, n, t.dt, every, params)
    fwd = time.perf_counter() - w0
    w0 = time.perf_counter()
    gr, ge = s.adjoint_backward(sv)
    bwd = time.perf_counter() - w0
    launches = s.launch_count() - l0
    sv.free()
    s.close()
    out = {"forward_s": fwd, "backward_s": bwd, "backward_over_forward": bwd / fwd, "loss": loss,
           "steps": n, "checkpoint_every": every, "parameters": 2 * t.n_elems,
           "grad_norm": {"rate": float(np.linalg.norm(gr)), "logE": float(np.linalg.norm(ge))},
           "gpu_launches": launches}
    if fd_dirs:
        ts = api.Solver(t, newton_tol=1e-11, krylov_rtol=1e-13)

        def lossf(r, e):
            ts.set_positions(t.pos)
            lv, sp = ts.adjoint_forward(r, e, n, t.dt, every, params)
            sp.free()
            return lv

        ts.set_positions(t.pos)
        _, sv = ts.adjoint_forward(rate, logE, n, t.dt, every, params)
        gt_r, gt_e = ts.adjoint_backward(sv)
        sv.free()
        rng = np.random.default_rng(seed)
        checks = []
        for k in range(fd_dirs):
            d = rng.standard_normal(t.n_elems)
            if k % 2 == 0:
                h = 1e-3 * np.abs(rate).max()
                f = (lossf(rate + h * d, logE) - lossf(rate - h * d, logE)) / (2 * h)
                adj = float(gt_r @ d)
            elif fd_order4:
                # fourth-order central difference at h = 1e-2: the derivative
                # along log E is small against the loss, so a 2-point step small
                # enough for its truncation leaves it in the loss's noise
                h = 1e-2
                f = (-lossf(rate, logE + 2 * h * d) + 8 * lossf(rate, logE + h * d)
                     - 8 * lossf(rate, logE - h * d) + lossf(rate, logE - 2 * h * d)) / (12 * h)
                adj = float(gt_e @ d)
            else:
                h = 1e-4
                f = (lossf(rate, logE + h * d) - lossf(rate, logE - h * d)) / (2 * h)
                adj = float(gt_e @ d)
            c6 = {}
            if k < fd_h6:
                # the same direction at h = 1e-6 relative (rates: 1e-6 x the
                # largest rate; log E: 1e-6), where the loss's rounding shows
                h6 = (1e-6 * np.abs(rate).max()) if k % 2 == 0 else 1e-6
                if k % 2 == 0:
                    f6 = (lossf(rate + h6 * d, logE) - lossf(rate - h6 * d, logE)) / (2 * h6)
                else:
                    f6 = (lossf(rate, logE + h6 * d) - lossf(rate, logE - h6 * d)) / (2 * h6)
                c6 = {"fd_h1e-6": f6, "rel_h1e-6": abs(adj - f6) / max(abs(f6), 1e-300)}
            checks.append({"parameter": "rate" if k % 2 == 0 else "logE", "adjoint": adj, "fd": f,
                           "rel": abs(adj - f) / max(abs(f), 1e-300), **c6})
        ts.close()
        out["fd"] = {"directions": fd_dirs,
                     "h": "rates: 1e-3 x the largest rate (2-point); log E: " +
                          ("1e-2 (4-point)" if fd_order4 else "1e-4 (2-point)"),
                     "solves": "Newton |du| <= 1e-11, Krylov relative residual 1e-13",
                     "max_rel_err": max(c["rel"] for c in checks), "checks": checks}
        if fd_h6:
            out["fd"]["max_rel_err_h1e-6"] = max(c["rel_h1e-6"] for c in checks if "rel_h1e-6" in c)
    return out


def adjoint_fd_sheet(cells=20, n=50, every=10, dirs=32, h=1e-2, seed=4321):
    """The adjoint against central differences along `dirs` seeded
    directions, alternating growth rates and log E, on a 20 x 20-cell sheet
    of the 320k-prism sheet's kind (4 layers, 3,200 prisms, log-normal E,
    internal viscosity 100, Gaussian growth bump) with the same loss, 50
    steps and checkpoints every 10.  Every solve is tight (Newton |du| <=
    1e-11, Krylov 1e-13, multigrid) and assembly deterministic.  A converged
    forward run is a function of its parameters only to ~1e-12 in the
    positions (the Newton test stops at |du| <= 1e-11), which 2-point
    differences at h = 1e-6 amplify to up to ~1e-4 of the derivative along
    log E; fourth-order differences at h = 1e-2 (rates: 1e-2 x the largest
    rate) bring that noise to ~1e-8 with O(h^4) truncation."""
    from tissuefolding_paperversion_gb300 import api, mesh

    t = mesh.config_large(seed=7, cells=cells)
    xy = t.pos.reshape(-1, 3)[:, :2]
    c = 0.5 * (xy.min(axis=0) + xy.max(axis=0))
    params = np.array([c[0], c[1], 5.0, 40.0])
    rate = t.rates.reshape(-1, 3)[:, 0].copy()
    logE = np.log(t.E)
    w0 = time.perf_counter()
    with api.Solver(t, newton_tol=1e-11, krylov_rtol=1e-13, deterministic=True, precond=2) as s:
        def lossf(r, e):
            s.set_positions(t.pos)
            lv, sp = s.adjoint_forward(r, e, n, t.dt, every, params)
            sp.free()
            return lv

        s.set_positions(t.pos)
        loss, sv = s.adjoint_forward(rate, logE, n, t.dt, every, params)
        gr, ge = s.adjoint_backward(sv)
        sv.free()
        rng = np.random.default_rng(seed)
        rel = []
        for k in range(dirs):
            d = rng.standard_normal(t.n_elems)
            if k % 2 == 0:
                hr = h * np.abs(rate).max()
                f = lambda a: lossf(rate + a * hr * d, logE)
                scale, adj = hr, float(gr @ d)
            else:
                f = lambda a: lossf(rate, logE + a * h * d)
                scale, adj = h, float(ge @ d)
            fd = (-f(2) + 8 * f(1) - 8 * f(-1) + f(-2)) / (12 * scale)
            rel.append(abs(adj - fd) / max(abs(fd), 1e-300))
    return {"prisms": t.n_elems, "steps": n, "checkpoint_every": every, "directions": dirs,
            "h": f"{h:g} (rates: {h:g} x the largest rate), 4-point central",
            "solves": "Newton |du| <= 1e-11, Krylov relative residual 1e-13, multigrid, deterministic assembly",
            "loss": loss, "max_rel_err": max(rel), "median_rel_err": float(np.median(rel)),
            "rel_err_rate": rel[0::2], "rel_err_logE": rel[1::2], "wall_s": time.perf_counter() - w0}


def run_adjoint(args, t):
    """The adjoint workload on its own (see adjoint_measure)."""
    n, every = args.adj_steps, args.adj_every
    r = adjoint_measure(t, n, every, args.adj_fd, fd_h6=args.adj_fd_h6, fd_order4=args.adj_fd_order4)
    print(json.dumps({
        "metric": "adjoint backward / forward cost", "value": r["backward_over_forward"], "unit": "ratio",
        "n_gpus": 1, "steps": n, "warmup": 1, "ms_per_step": (r["forward_s"] + r["backward_s"]) / n * 1e3,
        "higher_is_better": False, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"adjoint-{t.name}", "prisms": t.n_elems, "steps": n, "checkpoint_every": every,
                   "loss": "sum over apical nodes (z - 5 exp(-r^2/(2 40^2)))^2", "parameters": 2 * t.n_elems},
        **r,
    }))


def run_packing(args):
    """Implicit packing between two facing sheets: the per-step couple
    detection (the reference's O(N^2) detectPacingNodes) and the packing terms
    of an assembly, on the GPU; the CPU baseline is the restatement of the
    reference's scan timed on a sample of first nodes."""
    from tissuefolding_paperversion_gb300 import api, mesh

    t = mesh.config_facing_sheets(seed=0, n=args.pack_n, gap=1.5, E=100000.0)
    nn = t.n_nodes
    times = {}
    with api.Solver(t, precond=1) as s:
        s.set_positions(t.pos)
        for pack in (False, True):
            s.set_packing(pack)
            for _ in range(args.warmup):
                s.begin_step(t.dt)
            w = []
            a = []
            for _ in range(args.steps):
                w0 = time.perf_counter()
                s.begin_step(t.dt)            # synchronous: detection reads the couple count back
                w.append(time.perf_counter() - w0)
                s.set_state(t.pos, t.pos, t.dt)
                s.residual()
                w0 = time.perf_counter()
                s.assemble()
                s.residual()                   # waits for the assembly
                a.append(time.perf_counter() - w0)
            times[pack] = (float(np.median(w)), float(np.median(a)))
        pk = s.packing()
        l0 = s.launch_count()
        s.begin_step(t.dt)
        launches = s.launch_count() - l0
    # one implicit step with packing on the default preconditioner (the
    # multigrid, whose coarse levels carry the couples' blocks)
    with api.Solver(t) as s:
        s.set_growth_rates(t.rates)
        s.set_packing(True)
        st = s.newton_step(t.dt)
        mg = s.multigrid_info()[0]
    step = {"ms": st["ms_total"], "newton_iters": st["iters"], "krylov_iters": st["krylov_total"],
            "converged": st["converged"], "preconditioner": "smoothed-aggregation multigrid "
            + "/".join(map(str, mg)) if mg else "block-Jacobi"}
    detect_s = times[True][0] - times[False][0]
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import packing as op
        vref = op.reference_volumes(t.pos.reshape(-1, 3)[t.conn.reshape(-1, 6)])
        m = op.node_masses(t.conn, nn, vref, np.tile(np.eye(3), (t.n_elems, 1, 1)))
        elig = np.flatnonzero((m != 0) & ((t.node_placement == 0) | (t.node_placement == 1)))
        sample = np.random.default_rng(0).choice(elig, size=min(400, elig.size), replace=False)
        sample.sort()
        nb = op.neighbours(t.conn, nn)
        w0 = time.perf_counter()
        op.detect(t.pos, t.conn, t.node_placement, m, True, masters=sample, nb=nb)
        per = (time.perf_counter() - w0) / sample.size
        full_s = per * elig.size
        cpu = {"value": nn / full_s, "unit": "nodes/s", "cores": 1, "kind": "port",
               "sample": f"O(N^2) scan (numpy over the partners of each first node) from {sample.size} of "
                         f"{elig.size} eligible first nodes, {per * sample.size:.1f} s; full scan estimated "
                         f"{full_s:.0f} s"}
    print(json.dumps({
        "metric": "packing couple detection, nodes/s", "value": nn / detect_s, "unit": "nodes/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": detect_s * 1e3, "higher_is_better": True,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"packing-facing-sheets-{t.n_elems}", "nodes": nn, "prisms": t.n_elems,
                   "gap_um": 1.5, "couples": int(len(pk["nodes"])), "detect_distance_um": pk["detect"]},
        "detection_ms": detect_s * 1e3,
        "packing_assembly_ms": (times[True][1] - times[False][1]) * 1e3,
        "newton_step_with_packing": step,
        "begin_step_ms": {"without": times[False][0] * 1e3, "with": times[True][0] * 1e3},
        "timing": "host wall clock around synchronous calls, median of the timed steps",
        "gpu_launches": launches,
        "cpu_baseline": cpu,
    }))


def growth_functions_for(t):
    """A uniform function turned in the xy plane in the apical half, a ring
    and a grid function over the sheet, as a model file would set them."""
    from tissuefolding_paperversion_gb300 import mesh

    p = t.pos.reshape(-1, 3)
    lo, hi = p.min(axis=0), p.max(axis=0)
    ra, aa = mesh.grid_growth_inputs(1, 12, 9, scale=2e-5)
    return [dict(kind="uniform", rates=[1e-5, 5e-6, 0.0], angle_rad=0.6, zmin=0.0, zmax=0.5),
            dict(kind="ring", centre=((lo[0] + hi[0]) / 2, (lo[1] + hi[1]) / 2), inner_radius=0.1 * (hi[0] - lo[0]),
                 outer_radius=0.45 * (hi[0] - lo[0]), rates=[2e-5, 2e-5, 0.0], angle_rad=0.0),
            dict(kind="grid", rates=ra, angles_deg=aa)]


def run_growth(args, t):
    """The per-step growth update with growth functions of the three reference
    types (uniform, ring, grid on the current shape) against the per-element
    rates alone, on the start shape and on the sheet turned by 20 degrees
    (where every prism's growth is turned with it); the CPU baseline is the
    numpy restatement of the reference's calculateGrowth on the same sheet."""
    from tissuefolding_paperversion_gb300 import api

    fns = growth_functions_for(t)
    # the sheet turned by 20 degrees about z (its centre): every prism's deformation
    # gradient is then a rotation, so every prism runs the polar iteration of the turn
    p = t.pos.reshape(-1, 3)
    c = 0.5 * (p.min(axis=0) + p.max(axis=0))
    ang = np.deg2rad(20.0)
    R = np.array([[np.cos(ang), -np.sin(ang), 0.0], [np.sin(ang), np.cos(ang), 0.0], [0.0, 0.0, 1.0]])
    turned = ((p - c) @ R.T + c).reshape(-1)
    times = {}
    with api.Solver(t) as s:
        s.set_growth_rates(t.rates)
        for key in ("rates", "functions", "functions_turned"):
            if key == "functions":
                for f in fns:
                    kw = {k: v for k, v in f.items() if k != "kind"}
                    getattr(s, "add_" + f["kind"] + "_growth")(**kw)
            s.set_positions(turned if key == "functions_turned" else t.pos)
            for _ in range(args.warmup):
                s.begin_step(t.dt)
                s.end_step()
            w = []
            for _ in range(max(args.steps, 5)):
                w0 = time.perf_counter()
                s.begin_step(t.dt)
                s.end_step()                   # synchronises the stream
                w.append(time.perf_counter() - w0)
            times[key] = float(np.median(w))
        l0 = s.launch_count()
        s.begin_step(t.dt)
        s.end_step()
        launches = s.launch_count() - l0
    times[False], times[True] = times["rates"], times["functions"]
    extra_s = max(times[True] - times[False], 1e-9)
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import growth as og
        o = og.GrowthOracle(t.pos, t.conn, t.node_placement)
        og.add_functions(o, fns)
        w0 = time.perf_counter()
        o.grow(np.eye(3), t.pos, 0.0, t.dt, t.rates)
        cpu_s = time.perf_counter() - w0
        cpu = {"value": t.n_elems / cpu_s, "unit": "prisms/s", "cores": 1, "kind": "port",
               "sample": f"numpy restatement of calculateGrowth on all {t.n_elems} prisms, {cpu_s:.2f} s"}
    print(json.dumps({
        "metric": "growth update with uniform + ring + grid functions, prisms/s", "value": t.n_elems / times[True],
        "unit": "prisms/s", "n_gpus": 1, "steps": max(args.steps, 5), "warmup": args.warmup,
        "ms_per_step": times[True] * 1e3, "higher_is_better": True, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"growth-functions-{t.n_elems}", "prisms": t.n_elems, "nodes": t.n_nodes,
                   "functions": [f["kind"] for f in fns]},
        "begin_step_ms": {"rates_only": times[False] * 1e3, "with_functions": times[True] * 1e3,
                          "with_functions_turned_sheet": times["functions_turned"] * 1e3},
        "functions_extra_ms": extra_s * 1e3,
        "functions_extra_ms_turned_sheet": (times["functions_turned"] - times[False]) * 1e3,
        "shapes": "with_functions: the start shape (no prism turned: the polar iteration is skipped); "
                  "turned_sheet: the sheet turned by 20 degrees (every prism runs the polar iteration)",
        "timing": "host wall clock around begin_step + end_step (synchronous), median of the timed steps",
        "gpu_launches": launches,
        "cpu_baseline": cpu,
    }))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="large", choices=["large", "medium", "small", "wing"])
    ap.add_argument("--workload", default="plain", choices=["plain", "batch", "adjoint", "packing", "growth"],
                    help="plain: the 320k-prism Newton step; batch: the 256-instance sweep; "
                         "adjoint: gradient of an apical shape loss through n steps; "
                         "packing: couple detection between two facing sheets; "
                         "growth: the per-step growth update with uniform, ring and grid functions")
    ap.add_argument("--pack-n", type=int, default=200, help="nodes per side of each sheet (packing workload)")
    ap.add_argument("--adj-steps", type=int, default=50)
    ap.add_argument("--adj-every", type=int, default=10)
    ap.add_argument("--adj-fd", type=int, default=0, help="central-difference checks along random directions")
    ap.add_argument("--adj-fd-order4", action="store_true",
                    help="log E directions by a fourth-order central difference at h = 1e-2")
    ap.add_argument("--adj-fd-h6", type=int, default=0,
                    help="of those directions, how many are also differenced at h = 1e-6 relative")
    ap.add_argument("--instances", type=int, default=256)
    ap.add_argument("--mode", default="step", choices=["step", "assembly"],
                    help="step: Newton steps (the bench); assembly: back-to-back K+f assemblies only")
    ap.add_argument("--ref-seconds", type=float, default=6.0,
                    help="CPU seconds per timed reference step and per CPU-baseline sample")
    ap.add_argument("--quick", action="store_true",
                    help="plain workload only: leave out the 1,600-prism, batch and adjoint sub-measurements")
    ap.add_argument("--adj-fd-default", type=int, default=2,
                    help="central-difference directions of the adjoint sub-measurement of the plain workload")
    ap.add_argument("--precond", type=int, default=0,
                    help="0 auto (smoothed-aggregation multigrid from 20,000 nodes), 1 block-Jacobi, "
                         "2 smoothed-aggregation multigrid, 3 plain-aggregation multigrid")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mg-reuse", type=int, default=0,
                    help="plain workload: keep the multigrid's coarse levels for up to this many steps "
                         "(tf_options.multigrid_reuse_steps; 0: the library's default, 4; negative: "
                         "rebuild at every step)")
    ap.add_argument("--host-loops", action="store_true",
                    help="host-checked Krylov chunks and host-driven Newton iterations instead of the device-side "
                         "while loops (ncu cannot see kernels inside conditional graph nodes)")
    args = ap.parse_args()
    from tissuefolding_paperversion_gb300 import mesh

    if args.workload == "batch":
        run_batch(args)
        return
    if args.workload == "packing":
        run_packing(args)
        return
    if args.config == "large":
        t = mesh.config_large(seed=0)
    elif args.config == "wing":
        t = mesh.config_wing(seed=0)
    elif args.config == "medium":
        t = mesh.config_large(seed=0, cells=130)
    else:
        t = mesh.config_small(seed=0)
    if args.mode == "assembly" and args.impl == "ours":
        run_assembly_only(args, t)
        return
    if args.workload == "adjoint":
        run_adjoint(args, t)
        return
    if args.workload == "growth":
        run_growth(args, t)
        return
    if args.impl == "reference":
        run_reference(args, t)
    else:
        run_gpu(args, t)


if __name__ == "__main__":
    main()
