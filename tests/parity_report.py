"""Error of the CUDA path against the FP64 oracle, per benchmark configuration.

    python tests/parity_report.py [--quick]

Prints one JSON object per configuration and a markdown table.  Sizes where the
oracle can run the whole case are compared step by step; at full size the
checks are size-independent (sampled element tangents, the oracle's residual of
the GPU's converged state, the value-filtered CSR pattern).  The oracle is the
project's C restatement of the reference's algorithm (oracle/), pinned to the
reference's own sources by tests/test_oracle.py and tests/golden/.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle.oracle import CLOSED, LITERAL, Port, build_port  # noqa: E402
from tissuefolding_paperversion_gb300 import api, mesh  # noqa: E402

GOLD = os.path.join(ROOT, "tests", "golden")


def force_scale(t):
    p = t.pos.reshape(-1, 3)
    c = t.conn.reshape(-1, 6)
    return float(np.max(t.E)) * float(np.mean(np.sum((p[c[:, 1]] - p[c[:, 0]]) ** 2, axis=1)))


def rel(a, b):
    s = np.abs(b).max()
    return float(np.abs(a - b).max() / (s if s > 0 else 1.0))


def config1(precond):
    f = np.load(os.path.join(GOLD, "steps_small.npz"))
    t = mesh.config_small(seed=0)
    err, same = 0.0, True
    with api.Solver(t, precond=precond) as s:
        s.set_growth_rates(t.rates)
        for k in range(f["positions"].shape[0]):
            out = s.newton_step(t.dt)
            err = max(err, rel(s.positions(), f["positions"][k]))
            same &= out["iters"] == f["iters"][k]
    return {"config": f"1: {t.n_elems} prisms, 20 steps, {'multigrid' if precond == 2 else 'block-Jacobi'}",
            "positions_max_rel_err": err, "newton_iters_identical": bool(same),
            "against": "reference-generated golden positions (tests/golden/steps_small.npz)"}


def full_size(t, label, csr=True, samples=64):
    t0 = time.time()
    with api.Solver(t) as s:
        s.set_growth_rates(t.rates)
        out = s.newton_step(t.dt)
        pos = s.positions()
        Fg, _ = s.get_Fg()
        un = t.pos
        s.set_state(pos, un, t.dt)
        s.assemble()
        g_gpu = s.residual()
        if csr:
            ia, ja, a = s.export_csr(1e-13)
        area = s.viscosity_surfaces()
        rng = np.random.default_rng(0)
        sample = np.sort(rng.choice(t.n_elems, samples, replace=False))
        got = [s.element_eval(int(e), 1) for e in sample]
    p = Port(t)
    p.set_Fg(Fg)
    p.set_viscosity_surfaces(area)
    g_cpu = p.residual(pos, un, t.dt)
    fs = force_scale(t)
    ek = ef = 0.0
    for e, r in zip(sample, got):
        ref = p.element_eval(pos, un, t.dt, LITERAL, int(e), 1)
        ek = max(ek, rel(r["Ke"], ref["Ke"]), rel(r["Kv"], ref["Kv"]))
        ef = max(ef, float(np.abs(r["fe"] - ref["fe"]).max()) / fs, float(np.abs(r["fv"] - ref["fv"]).max()) / fs)
    res = {"config": label, "newton_iters": out["iters"], "last_dunorm": float(out["dunorm"][-1]),
           "residual_gpu_vs_oracle_over_force_scale": float(np.abs(g_gpu - g_cpu).max()) / fs,
           "oracle_residual_of_gpu_state_over_force_scale": float(np.abs(g_cpu).max()) / fs,
           "sampled_element_K_max_rel_err": ek, "sampled_element_f_max_err_over_force_scale": ef,
           "element_samples": samples}
    if csr:
        p.assemble(pos, un, t.dt, CLOSED)
        ia2, ja2, a2 = p.export_filtered(1e-13)
        same = ia.shape == ia2.shape and np.array_equal(ia, ia2) and np.array_equal(ja, ja2)
        res["csr_pattern_bit_exact"] = bool(same)
        res["csr_nnz"] = int(ia[-1])
        if same:
            res["K_max_rel_err"] = rel(a, a2)
    res["seconds"] = time.time() - t0
    return res


def config4(n=8):
    ts = [mesh.config_batch_instance(s) for s in range(n)]
    with api.Batch(ts) as b:
        b.set_growth_rates()
        for _ in range(2):
            b.step(ts[0].dt)
        pos = [b.instance_positions(i).copy() for i in range(n)]
    worst = 0.0
    for i, t in enumerate(ts):
        with api.Solver(t) as s:
            s.set_growth_rates(t.rates)
            for _ in range(2):
                s.newton_step(t.dt)
            worst = max(worst, rel(pos[i], s.positions()))
    # the smallest instance against the oracle's Newton steps
    k = int(np.argmin([t.n_elems for t in ts]))
    t = ts[k]
    p = Port(t)
    for _ in range(2):
        p.step(t.dt, t.rates)
    return {"config": f"4: first {n} of the 256 batch instances ({sum(t.n_elems for t in ts)} prisms), 2 steps",
            "batched_vs_plain_max_rel_err": worst,
            "smallest_instance_vs_oracle_max_rel_err": rel(pos[k], p.positions()),
            "smallest_instance_prisms": t.n_elems}


def config5():
    t = mesh.config_tiny(seed=5, n=7, n_layers=3, eta=100.0)
    rng = np.random.default_rng(105)
    rate = 1e-4 * (1.0 + 0.5 * rng.uniform(-1, 1, t.n_elems))
    logE = np.log(t.E)
    xy = t.pos.reshape(-1, 3)
    c = xy[:, :2].mean(axis=0)
    params = np.array([c[0], c[1], 1.2 * xy[t.node_placement == 1, 2].mean(), 8.0])
    n, every = 4, 2

    def oracle_loss(r, e):
        t2 = mesh.Tissue(**{**t.__dict__, "E": np.exp(e)})
        r3 = np.zeros((t.n_elems, 3))
        r3[:, 0] = r
        r3[:, 1] = r
        p = Port(t2)
        for _ in range(n):
            p.step(t.dt, r3.reshape(-1))
        x = p.positions().reshape(-1, 3)[t.node_placement == 1]
        f = params[2] * np.exp(-((x[:, 0] - params[0]) ** 2 + (x[:, 1] - params[1]) ** 2) / (2 * params[3] ** 2))
        return float(np.sum((x[:, 2] - f) ** 2))

    with api.Solver(t, newton_tol=1e-10, krylov_rtol=1e-12, deterministic=True) as s:
        def gpu_loss(r, e):
            s.set_positions(t.pos)
            lv, sv = s.adjoint_forward(r, e, n, t.dt, every, params)
            sv.free()
            return lv
        s.set_positions(t.pos)
        _, sv = s.adjoint_forward(rate, logE, n, t.dt, every, params)
        gr, ge = s.adjoint_backward(sv)
        sv.free()
        worst_gpu = worst_ora = 0.0
        for _ in range(4):
            d = rng.standard_normal(t.n_elems)
            for g, h, args in ((gr, 1e-3 * np.abs(rate).mean(), "rate"), (ge, 1e-4, "logE")):
                def shift(sg):
                    return (rate + sg * h * d, logE) if args == "rate" else (rate, logE + sg * h * d)
                adj = float(g @ d)
                fd_g = (gpu_loss(*shift(1)) - gpu_loss(*shift(-1))) / (2 * h)
                fd_o = (oracle_loss(*shift(1)) - oracle_loss(*shift(-1))) / (2 * h)
                worst_gpu = max(worst_gpu, abs(adj - fd_g) / abs(fd_g))
                worst_ora = max(worst_ora, abs(adj - fd_o) / abs(fd_o))
    return {"config": f"5 (reduced): adjoint, {t.n_elems} prisms, {n} steps, checkpoints every {every}, "
                      "4 directions x 2 parameter sets",
            "adjoint_vs_gpu_central_differences_max_rel_err": worst_gpu,
            "adjoint_vs_oracle_central_differences_max_rel_err": worst_ora}


def packing(name, kw, precond):
    """Implicit packing: steps with packing against the reference's own
    classes (fixtures tests/golden/steps_facing_packing*.npz)."""
    f = np.load(os.path.join(GOLD, name + ".npz"))
    t = mesh.config_facing_sheets(**kw)
    off = np.concatenate([[0], np.cumsum(f["pk_n"])])
    err, same, couples = 0.0, True, True
    with api.Solver(t, krylov_rtol=1e-12, precond=precond) as s:
        s.set_growth_rates(t.rates)
        s.set_packing(True, reference_merge=bool(f["drop_last_segment"]))
        for k in range(f["positions"].shape[0]):
            out = s.newton_step(t.dt)
            err = max(err, rel(s.positions(), f["positions"][k]))
            same &= out["iters"] == f["iters"][k]
            couples &= bool(np.array_equal(s.packing()["nodes"], f["pk_nodes"][off[k]:off[k + 1]]))
    return {"config": f"f3 packing: {name} ({t.n_elems} prisms, {f['positions'].shape[0]} steps), "
                      f"{'multigrid' if precond == 2 else 'block-Jacobi'}",
            "positions_max_rel_err": err, "newton_iters_identical": bool(same), "couples_identical": couples}


def growth(name):
    """Growth functions: steps with the reference's growth functions against its
    own growth-function classes (fixtures tests/golden/steps_grid_growth*.npz,
    steps_growth_functions.npz, steps_growth_rotated.npz)."""
    from oracle import growth as og

    f = np.load(os.path.join(GOLD, name + ".npz"))
    start, interp, pinned = None, 1, False
    if name == og.MIXED_FIXTURE:
        t, fns = og.mixed_case()
    elif name == og.ROTATED_FIXTURE:
        t, start, fns = og.rotated_case()
    else:
        t, fns, interp, pinned = og.fixture_case(name)
    err, fg, same = 0.0, 0.0, True
    with api.Solver(t, krylov_rtol=1e-12) as s:
        og.add_functions(s, fns)
        s.set_grid_growth_mode(interp, pinned)
        s.set_growth_rates(t.rates)
        if start is not None:
            s.set_positions(start)
        for k in range(f["positions"].shape[0]):
            out = s.newton_step(t.dt)
            err = max(err, rel(s.positions(), f["positions"][k]))
            fg = max(fg, float(np.abs(s.get_Fg()[0] - f["Fg"][k]).max()))
            same &= out["iters"] == f["iters"][k]
    return {"config": f"f1 growth functions: {name} ({t.n_elems} prisms, {f['positions'].shape[0]} steps)",
            "positions_max_rel_err": err, "Fg_max_abs_err": fg, "newton_iters_identical": bool(same)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--quick", action="store_true", help="skip the 1.0M-prism wing")
    ap.add_argument("--only-f", action="store_true", help="only the rows of the next-step features (f1, f3)")
    args = ap.parse_args()
    build_port()
    runs = []
    if not args.only_f:
        runs += [lambda: config1(1), lambda: config1(2),
                 lambda: full_size(mesh.config_large(seed=0), "2: 320,000 prisms, first Newton step")]
        if not args.quick:
            runs.append(lambda: full_size(mesh.config_wing(seed=0), "3: 995,824-prism wing, first Newton step",
                                          csr=False))
        runs += [config4, config5]
    for name, kw in (("steps_facing_packing", dict(seed=12, gap=1.5, E=100000.0, eta=0.0)),
                     ("steps_facing_packing_viscous", dict(seed=13, gap=1.5, E=100000.0, eta=100.0))):
        runs += [lambda name=name, kw=kw, pc=pc: packing(name, kw, pc) for pc in (1, 2)]
    for name in ("steps_grid_growth", "steps_grid_growth_pinned", "steps_growth_functions", "steps_growth_rotated"):
        runs.append(lambda name=name: growth(name))
    out = []
    for r in runs:
        out.append(r())
        print(json.dumps(out[-1]), flush=True)
    print()
    for o in out:
        print("| " + o["config"] + " | " + "; ".join(f"{k} = {v:.3g}" if isinstance(v, float) else f"{k} = {v}"
                                                     for k, v in o.items() if k != "config") + " |")


if __name__ == "__main__":
    main()
