"""The reference's mesh files on the host side of the GPU step.

`load_tissue` reads a reference .mesh input file (through the library's
`tf_read_mesh_file`) into a `Tissue`, with the boundary conditions and
material the modelinput file would otherwise set (basal nodes fixed in z,
external viscosity on the apical and basal surfaces, uniform material).
`write_mesh_file` writes a tissue in the same input format, and
`api.write_frame` writes save frames the reference's viewer reads.
"""
from __future__ import annotations

import numpy as np

from . import api, mesh


def write_mesh_file(path, t: "mesh.Tissue", tissue_type=None, at_circumference=None):
    """A tissue in the .mesh input format (Simulation.cpp:2074-2239): nodes
    with placement / type / circumference flags, prisms (shape type 1) with
    their node ids and reference positions, and no tissue weights."""
    pos = t.pos.reshape(-1, 3)
    conn = t.conn.reshape(-1, 6)
    n = pos.shape[0]
    ty = np.zeros(n, dtype=int) if tissue_type is None else np.asarray(tissue_type)
    ci = np.zeros(n, dtype=int) if at_circumference is None else np.asarray(at_circumference)
    with open(path, "w") as f:
        f.write(f"{n}\n")
        for i in range(n):
            f.write(f"{pos[i, 0]:.17g} {pos[i, 1]:.17g} {pos[i, 2]:.17g} {int(t.node_placement[i])} "
                    f"{int(ty[i])} {int(ci[i])}\n")
        f.write(f"{conn.shape[0]}\n")
        refs = (pos[conn].reshape(-1, 18) if getattr(t, "ref_pos", None) is None
                else np.asarray(t.ref_pos, dtype=np.float64).reshape(-1, 18))
        for e in range(conn.shape[0]):
            ids = " ".join(str(int(v)) for v in conn[e])
            ref = " ".join(f"{v:.17g}" for v in refs[e])
            f.write(f"1 {ids} {ref}\n")
        f.write("0\n")


def load_tissue(path, E=1000.0, nu=0.3, eta=0.0, ext_visc=10.0, dt=60.0, rates=None, name=None):
    """A `Tissue` from a reference .mesh file.  The file gives the geometry,
    the node placement (0 basal, 1 apical, 2 middle, 3 lateral), the prism
    connectivity and each prism's reference (stress-free) shape; the rest
    takes the values given here."""
    m = api.read_mesh_file(path)
    n = m["placement"].size
    e = m["conn"].size // 6
    pl = m["placement"].astype(np.int32)
    t = mesh.Tissue(pos=m["pos"], conn=m["conn"], fixed=mesh._bc_basal_z_fixed(pl),
                    ext_visc=mesh._ext_visc_surfaces(pl, ext_visc, ext_visc), node_placement=pl,
                    E=np.full(e, float(E)), nu=np.full(e, float(nu)), eta=np.full(e, float(eta)),
                    rates=np.zeros(3 * e) if rates is None else np.asarray(rates, dtype=np.float64),
                    dt=dt, name=name or f"mesh-{e}", ref_pos=m["ref_pos"])
    info = {"tissue_type": m["tissue_type"], "at_circumference": m["at_circumference"], "ref_pos": m["ref_pos"],
            "n_nodes": n, "n_elems": e}
    return t, info
