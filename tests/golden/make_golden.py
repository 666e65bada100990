"""Generates the golden fixtures under tests/golden from the reference itself.

Run where the reference checkout is present (it builds oracle/_ref from the
reference's own sources with the project-written GSL/uBLAS/Pardiso
stand-ins):

    python tests/golden/make_golden.py [--only-bound | --only-packing | --only-grid]

Every fixture records the seeded inputs that produced it, so tests rebuild
the same inputs with tissuefolding_paperversion_gb300.mesh and compare.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import growth as og  # noqa: E402
from oracle.oracle import Ref  # noqa: E402
from tissuefolding_paperversion_gb300 import mesh  # noqa: E402


def element_fixture(name, eta, seed):
    t = mesh.config_tiny(seed=seed, n=3, n_layers=2, eta=eta)
    r = Ref(t)
    assert (r.conn() == t.conn).all()
    Fg = mesh.growth_Fg(t, seed=seed + 1)
    r.set_Fg(Fg)
    uk, un = mesh.perturbed_state(t, seed=seed + 2)
    ev = r.element_eval(uk, un, t.dt)
    r.set_positions(uk)
    area = r.update_viscosity_surfaces()
    ia, ja, a, g = r.assemble(uk, un, t.dt)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), seed=seed, eta=eta, Fg=Fg, uk=uk, un=un, dt=t.dt,
                        Ke=ev["Ke"], Kv=ev["Kv"], fe=ev["fe"], fv=ev["fv"], area=area, ia=ia, ja=ja, a=a, g=g)
    r.close()


def steps_fixture(name, t, n_steps, seed_note):
    r = Ref(t)
    assert (r.conn() == t.conn).all()
    pos, iters, dun = [], [], []
    t0 = time.time()
    for s in range(n_steps):
        out = r.step(t.dt, t.rates)
        pos.append(r.positions())
        iters.append(out["iters"])
        d = np.zeros(21)
        d[: len(out["dunorm"])] = out["dunorm"]
        dun.append(d)
    Fg, invFg = r.get_Fg()
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), positions=np.array(pos), iters=np.array(iters),
                        dunorm=np.array(dun), Fg=Fg, note=seed_note)
    r.close()
    return time.time() - t0


def bound_dofs(t):
    """Slave/master DOF couples for the binding fixture: x of two apical nodes
    that share an element, z of two apical nodes at opposite corners (not
    element neighbours), y of two middle-layer nodes."""
    pos = t.pos.reshape(-1, 3)
    ap = np.flatnonzero(t.node_placement == 1)
    mid = np.flatnonzero(t.node_placement == 2)
    c = t.conn.reshape(-1, 6)
    e0 = [e for e in range(c.shape[0]) if t.node_placement[c[e, 3]] == 1][0]
    a_lo = ap[np.argmin(pos[ap, 0] + pos[ap, 1])]
    a_hi = ap[np.argmax(pos[ap, 0] + pos[ap, 1])]
    slaves = [3 * c[e0, 4] + 0, 3 * a_hi + 2, 3 * mid[-1] + 1]
    masters = [3 * c[e0, 3] + 0, 3 * a_lo + 2, 3 * mid[0] + 1]
    return np.array(slaves, dtype=np.int32), np.array(masters, dtype=np.int32)


def bound_steps_fixture(name, t, n_steps, seed_note):
    r = Ref(t)
    s, m = bound_dofs(t)
    r.set_bindings(s, m)
    pos, iters = [], []
    for _ in range(n_steps):
        out = r.step(t.dt, t.rates)
        pos.append(r.positions())
        iters.append(out["iters"])
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), positions=np.array(pos), iters=np.array(iters),
                        slaves=s, masters=m, note=seed_note)
    r.close()


def packing_steps_fixture(name, t, n_steps, drop_last_segment, seed_note):
    """Steps with the reference's implicit packing (couples detected at each
    step start), plus the couples, node masses and one assembled system with
    its packing forces at a perturbed state of the first step."""
    r = Ref(t)
    r.set_packing(True, drop_last_segment)
    pos, iters, pk_nodes, pk_w, pk_mbar, pk_thr, pk_det, pk_n = [], [], [], [], [], [], [], []
    for _ in range(n_steps):
        out = r.step(t.dt, t.rates)
        p = r.packing()
        pk_n.append(len(p["nodes"]))
        pk_nodes.append(p["nodes"])
        pk_w.append(p["w"])
        pk_mbar.append(p["mbar"])
        pk_thr.append(p["threshold"])
        pk_det.append(p["detect"])
        pos.append(r.positions())
        iters.append(out["iters"])
    r.close()
    # one assembly at a perturbed state, couples detected at un
    r = Ref(t)
    r.set_packing(True, drop_last_segment)
    uk, un = mesh.perturbed_state(t, seed=7, amp=0.05)
    r.set_positions(un)
    r.pack_detect()
    p0 = r.packing()
    masses = r.node_masses()
    r.update_viscosity_surfaces()
    ia, ja, a, g = r.assemble(uk, un, t.dt)
    f = r.pack_forces()
    r.close()
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), positions=np.array(pos), iters=np.array(iters),
                        pk_n=np.array(pk_n), pk_nodes=np.concatenate(pk_nodes), pk_w=np.concatenate(pk_w),
                        pk_mbar=np.concatenate(pk_mbar), pk_threshold=np.array(pk_thr), pk_detect=np.array(pk_det),
                        asm_nodes=p0["nodes"], asm_w=p0["w"], asm_mbar=p0["mbar"], asm_threshold=p0["threshold"],
                        asm_masses=masses, asm_ia=ia, asm_ja=ja, asm_a=a, asm_g=g, asm_forces=f,
                        drop_last_segment=drop_last_segment, note=seed_note)


def packing_fixtures():
    # stiff sheets (E = 1e5 Pa): the reference's packing force (5000 x the
    # couple's mean node mass) deforms softer sheets by several µm per step
    # and makes later steps diverge
    t = mesh.config_facing_sheets(seed=12, gap=1.5, E=100000.0, eta=0.0)
    packing_steps_fixture("steps_facing_packing", t, 3, True,
                          "config_facing_sheets(seed=12, gap=1.5, E=1e5, eta=0), packing on, last segment dropped")
    t = mesh.config_facing_sheets(seed=13, gap=1.5, E=100000.0, eta=100.0)
    packing_steps_fixture("steps_facing_packing_viscous", t, 2, False,
                          "config_facing_sheets(seed=13, gap=1.5, E=1e5, eta=100), packing on, every segment kept")


def grid_growth_fixture(name, n_steps):
    """Bounding-box positions and one growth update at the initial shape,
    then Newton steps with the grid functions and the per-element rates."""
    t, fns, interp, pinned = og.fixture_case(name)
    r = Ref(t)
    og.add_functions(r, fns)
    r.set_grid_mode(interp, pinned)
    relz, rel0, rel = r.grid_positions()
    r.grow(t.dt, t.rates)
    Fg_grow = r.get_Fg()[0]
    r.close()
    r = Ref(t)
    og.add_functions(r, fns)
    r.set_grid_mode(interp, pinned)
    pos, iters, Fg = [], [], []
    for _ in range(n_steps):
        out = r.step(t.dt, t.rates)
        pos.append(r.positions())
        iters.append(out["iters"])
        Fg.append(r.get_Fg()[0])
    r.close()
    extra = {}
    for i, f in enumerate(fns):
        extra[f"fn{i}_rates"] = f["rates"]
        extra[f"fn{i}_angles"] = f["angles_deg"]
        extra[f"fn{i}_window"] = np.array([f["init_time"], f["end_time"], f["zmin"], f["zmax"]])
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), relz=relz, rel0=rel0, rel=rel, Fg_grow=Fg_grow,
                        positions=np.array(pos), iters=np.array(iters), Fg=np.array(Fg), interp=interp,
                        pinned=pinned, n_fns=len(fns), note=og.fixture_case.__doc__, **extra)


def growth_functions_fixture(n_steps):
    """Newton steps with uniform, ring and grid functions mixed (in their
    order) after the per-element rates, and one growth update at the initial
    shape."""
    t, fns = og.mixed_case()
    r = Ref(t)
    og.add_functions(r, fns)
    r.grow(t.dt, t.rates)
    Fg_grow = r.get_Fg()[0]
    r.close()
    r = Ref(t)
    og.add_functions(r, fns)
    pos, iters, Fg = [], [], []
    for _ in range(n_steps):
        out = r.step(t.dt, t.rates)
        pos.append(r.positions())
        iters.append(out["iters"])
        Fg.append(r.get_Fg()[0])
    r.close()
    np.savez_compressed(os.path.join(HERE, og.MIXED_FIXTURE + ".npz"), Fg_grow=Fg_grow, positions=np.array(pos),
                        iters=np.array(iters), Fg=np.array(Fg), note=og.mixed_case.__doc__)


def growth_rotated_fixture(n_steps):
    """Newton steps from a start shape turned by 20 degrees: the growth of
    every prism is turned with it (CalculateGrowthRotationByF)."""
    t, start, fns = og.rotated_case()
    r = Ref(t)
    og.add_functions(r, fns)
    r.set_positions(start)
    r.grow(t.dt, t.rates)
    Fg_grow = r.get_Fg()[0]
    r.close()
    r = Ref(t)
    og.add_functions(r, fns)
    r.set_positions(start)
    pos, iters, Fg = [], [], []
    for _ in range(n_steps):
        out = r.step(t.dt, t.rates)
        pos.append(r.positions())
        iters.append(out["iters"])
        Fg.append(r.get_Fg()[0])
    r.close()
    np.savez_compressed(os.path.join(HERE, og.ROTATED_FIXTURE + ".npz"), Fg_grow=Fg_grow, positions=np.array(pos),
                        iters=np.array(iters), Fg=np.array(Fg), note=og.rotated_case.__doc__)


def grid_fixtures():
    for name in og.FIXTURES:
        grid_growth_fixture(name, 3)
    growth_functions_fixture(3)
    growth_rotated_fixture(3)


def main():
    if "--only-grid" in sys.argv:
        grid_fixtures()
        return
    if "--only-packing" in sys.argv:
        packing_fixtures()
        return
    if "--only-bound" in sys.argv:
        t = mesh.config_tiny(seed=15, n=5, n_layers=2, eta=100.0)
        bound_steps_fixture("steps_tiny_bound", t, 4, "config_tiny(seed=15,n=5,n_layers=2,eta=100), bound_dofs(t)")
        return
    element_fixture("elem_tiny_elastic", 0.0, 11)
    element_fixture("elem_tiny_viscous", 100.0, 12)
    t = mesh.config_tiny(seed=13, n=4, n_layers=2, eta=0.0)
    print("tiny elastic steps", steps_fixture("steps_tiny_elastic", t, 5, "config_tiny(seed=13,n=4,n_layers=2,eta=0)"))
    t = mesh.config_tiny(seed=14, n=4, n_layers=2, eta=100.0)
    print("tiny viscous steps", steps_fixture("steps_tiny_viscous", t, 5, "config_tiny(seed=14,n=4,n_layers=2,eta=100)"))
    t = mesh.config_small(seed=0)
    print("small steps", steps_fixture("steps_small", t, t.n_steps, "config_small(seed=0)"))
    t = mesh.config_tiny(seed=15, n=5, n_layers=2, eta=100.0)
    bound_steps_fixture("steps_tiny_bound", t, 4, "config_tiny(seed=15,n=5,n_layers=2,eta=100), bound_dofs(t)")
    packing_fixtures()
    grid_fixtures()


if __name__ == "__main__":
    main()
