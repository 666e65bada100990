"""Seeded prism-mesh and tissue-configuration generator.

Produces the arrays that the reference reads from its ``.mesh`` file and
``modelinput`` file for the implicit step, in the reference's conventions:

* node order: all nodes of the basal surface first, then each higher layer
  (TissueFolding/ToolBox/MeshGeneration/2DEllipse/src/Ellipse.cpp:531-582
  writes layers bottom-up);
* prism node order: basal triangle (0, 1, 2) counter-clockwise seen from the
  apical side, then the apical triangle (3, 4, 5) above it
  (Prism::checkRotationConsistency3D, Prism.cpp:364-412, swaps 1<->2 and
  4<->5 otherwise);
* node placement 0 = basal, 1 = apical, 2 = mid (Node.h:33);
* DOF index = 3 * node + dim (NewtonRaphsonSolver.cpp:135-141).

Meshes are structured triangular grids (each square split along one
diagonal) extruded into prism layers; elliptical sheets keep the squares of
the grid whose four corners lie inside the ellipse.  The reference builds its
meshes with Shewchuk's Triangle; a structured generator with the same
ordering rules is enough for every workload this package measures.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

HOUR = 3600.0


@dataclasses.dataclass
class Tissue:
    """One tissue instance: mesh, boundary conditions, material, growth."""

    pos: np.ndarray            # (3N,) float64 node positions (µm)
    conn: np.ndarray           # (6E,) int32 prism connectivity
    fixed: np.ndarray          # (3N,) uint8 fixed-DOF flags (Node::FixedPos)
    ext_visc: np.ndarray       # (3N,) float64 external viscosity (Node::externalViscosity)
    node_placement: np.ndarray  # (N,) int32 0 basal / 1 apical / 2 mid
    E: np.ndarray              # (E,) Young's modulus (Pa)
    nu: np.ndarray             # (E,) Poisson ratio
    eta: np.ndarray            # (E,) internal viscosity (Pa s)
    rates: np.ndarray          # (3E,) growth rates per element (1/s), x y z
    dt: float = 60.0           # time step (s)
    n_steps: int = 20
    name: str = "tissue"
    ref_pos: np.ndarray = None  # (18E,) reference (stress-free) prism shapes; None: the node positions

    @property
    def n_nodes(self) -> int:
        return self.pos.size // 3

    @property
    def n_elems(self) -> int:
        return self.conn.size // 6

    def centroids(self) -> np.ndarray:
        p = self.pos.reshape(-1, 3)
        return p[self.conn.reshape(-1, 6)].mean(axis=1)


def _grid_triangles(mask_sq: np.ndarray, nx: int, ny: int):
    """Triangles of an (nx x ny)-node grid, for squares where mask_sq is True.

    Square (i, j) has corners p00=(i,j), p10=(i+1,j), p01=(i,j+1),
    p11=(i+1,j+1); it is split into (p00, p10, p11) and (p00, p11, p01), both
    counter-clockwise seen from +z.
    """
    ii, jj = np.nonzero(mask_sq)            # ii along x, jj along y
    order = np.lexsort((ii, jj))             # row-major by y then x
    ii, jj = ii[order], jj[order]
    p00 = jj * nx + ii
    p10 = p00 + 1
    p01 = p00 + nx
    p11 = p01 + 1
    t1 = np.stack([p00, p10, p11], axis=1)
    t2 = np.stack([p00, p11, p01], axis=1)
    tri = np.stack([t1, t2], axis=1).reshape(-1, 3)
    return tri


def _extrude(xy: np.ndarray, tri: np.ndarray, n_layers: int, thickness: float):
    """Extrude a triangulated surface into prism layers (basal layer first)."""
    ns = xy.shape[0]
    z = np.linspace(0.0, thickness, n_layers + 1)
    pos = np.zeros((n_layers + 1, ns, 3))
    pos[:, :, 0:2] = xy[None, :, :]
    pos[:, :, 2] = z[:, None]
    conn = []
    for layer in range(n_layers):
        lo = tri + layer * ns
        hi = tri + (layer + 1) * ns
        conn.append(np.concatenate([lo, hi], axis=1))
    conn = np.concatenate(conn, axis=0).astype(np.int32)
    placement = np.full((n_layers + 1, ns), 2, dtype=np.int32)
    placement[0, :] = 0
    placement[-1, :] = 1
    return pos.reshape(-1), conn.reshape(-1), placement.reshape(-1)


def _compact(xy: np.ndarray, tri: np.ndarray):
    """Drop grid nodes that no triangle uses, renumbering in order."""
    used = np.zeros(xy.shape[0], dtype=bool)
    used[tri.reshape(-1)] = True
    newid = -np.ones(xy.shape[0], dtype=np.int64)
    newid[used] = np.arange(int(used.sum()))
    return xy[used], newid[tri]


def rect_sheet(nx: int, ny: int, spacing: float, n_layers: int, thickness: float,
               jitter: float, rng: np.random.Generator):
    xs = np.arange(nx) * spacing
    ys = np.arange(ny) * spacing
    X, Y = np.meshgrid(xs, ys)               # (ny, nx): row-major by y
    xy = np.stack([X.reshape(-1), Y.reshape(-1)], axis=1)
    if jitter > 0:
        xy = xy + rng.uniform(-jitter, jitter, size=xy.shape)
    mask = np.ones((nx - 1, ny - 1), dtype=bool)
    tri = _grid_triangles(mask, nx, ny)
    return _extrude(xy, tri, n_layers, thickness)


def ellipse_sheet(a: float, b: float, spacing: float, n_layers: int, thickness: float,
                  jitter: float, rng: np.random.Generator):
    nx = int(math.ceil(2 * a / spacing)) + 1
    ny = int(math.ceil(2 * b / spacing)) + 1
    xs = -a + np.arange(nx) * spacing
    ys = -b + np.arange(ny) * spacing
    X, Y = np.meshgrid(xs, ys)
    inside = (X / a) ** 2 + (Y / b) ** 2 <= 1.0          # (ny, nx)
    ins = inside.T                                        # (nx, ny)
    mask = ins[:-1, :-1] & ins[1:, :-1] & ins[:-1, 1:] & ins[1:, 1:]
    xy = np.stack([X.reshape(-1), Y.reshape(-1)], axis=1)
    if jitter > 0:
        xy = xy + rng.uniform(-jitter, jitter, size=xy.shape)
    tri = _grid_triangles(mask, nx, ny)
    xy, tri = _compact(xy, tri)
    return _extrude(xy, tri, n_layers, thickness)


def _bc_basal_z_fixed(placement: np.ndarray) -> np.ndarray:
    fixed = np.zeros((placement.size, 3), dtype=np.uint8)
    fixed[placement == 0, 2] = 1
    return fixed.reshape(-1)


def _ext_visc_surfaces(placement: np.ndarray, apical: float, basal: float) -> np.ndarray:
    """Node::setExternalViscosity (Node.cpp:68-116) without inner-tissue
    extension: apical nodes take the apical value, basal nodes the basal one,
    mid nodes keep 0 (they carry no viscosity surface either)."""
    ev = np.zeros((placement.size, 3))
    ev[placement == 1, :] = apical
    ev[placement == 0, :] = basal
    return ev.reshape(-1)


def _elem_relative_z(pos: np.ndarray, conn: np.ndarray) -> np.ndarray:
    """ShapeBase::setInitialZPosition (ShapeBase.cpp:612-627): 0 apical, 1 basal."""
    p = pos.reshape(-1, 3)
    zmin, zmax = p[:, 2].min(), p[:, 2].max()
    c = p[conn.reshape(-1, 6)].mean(axis=1)[:, 2]
    r = 1.0 - (c - zmin) / (zmax - zmin)
    return np.clip(r, 0.0, 1.0)


def config_small(seed: int = 0) -> Tissue:
    """100 x 100 µm square disc, 10 µm thick, 21 x 21 node grid, 2 layers:
    1323 nodes, 1600 prisms.  E = 1000 Pa, nu = 0.3, no internal viscosity,
    external viscosity 10 on apical and basal surfaces, basal nodes fixed in z.
    Growth 0.01/hr in-plane everywhere plus 0.005/hr in the apical half.
    20 steps of 60 s."""
    rng = np.random.default_rng(seed)
    pos, conn, pl = rect_sheet(21, 21, 5.0, 2, 10.0, 0.5, rng)
    ne = conn.size // 6
    relz = _elem_relative_z(pos, conn)
    r = np.full(ne, 0.01 / HOUR)
    r = r + np.where(relz <= 0.5, 0.005 / HOUR, 0.0)
    rates = np.zeros((ne, 3))
    rates[:, 0] = r
    rates[:, 1] = r
    return Tissue(pos=pos, conn=conn, fixed=_bc_basal_z_fixed(pl),
                  ext_visc=_ext_visc_surfaces(pl, 10.0, 10.0), node_placement=pl,
                  E=np.full(ne, 1000.0), nu=np.full(ne, 0.3), eta=np.zeros(ne),
                  rates=rates.reshape(-1), dt=60.0, n_steps=20, name="small-1600")


def _gaussian_bump(cxy: np.ndarray, peak: float, centre, width: float) -> np.ndarray:
    d2 = ((cxy - np.asarray(centre)[None, :]) ** 2).sum(axis=1)
    return peak * np.exp(-d2 / (2.0 * width * width))


def config_large(seed: int = 0, cells: int = 200, n_layers: int = 4) -> Tissue:
    """200 x 200 cell grid (5 µm spacing, 1000 x 1000 µm), 4 layers of 5 µm:
    202005 nodes, 320000 prisms.  E log-normal (mean 1000 Pa, sigma 0.3) per
    element, nu = 0.3, internal viscosity 100 Pa s, external viscosity 10 on
    apical/basal surfaces, basal nodes fixed in z.  In-plane growth: a
    Gaussian bump of peak 0.02/hr with seeded centre and width.  20 steps of
    60 s."""
    rng = np.random.default_rng(seed)
    n = cells + 1
    pos, conn, pl = rect_sheet(n, n, 5.0, n_layers, 5.0 * n_layers, 0.5, rng)
    ne = conn.size // 6
    sigma = 0.3
    E = rng.lognormal(mean=math.log(1000.0) - 0.5 * sigma * sigma, sigma=sigma, size=ne)
    L = cells * 5.0
    centre = rng.uniform(0.25 * L, 0.75 * L, size=2)
    width = rng.uniform(0.1 * L, 0.25 * L)
    c = Tissue(pos=pos, conn=conn, fixed=_bc_basal_z_fixed(pl),
               ext_visc=_ext_visc_surfaces(pl, 10.0, 10.0), node_placement=pl,
               E=E, nu=np.full(ne, 0.3), eta=np.full(ne, 100.0), rates=np.zeros(3 * ne),
               dt=60.0, n_steps=20, name=f"large-{ne}")
    g = _gaussian_bump(c.centroids()[:, :2], 0.02 / HOUR, centre, width)
    rates = np.zeros((ne, 3))
    rates[:, 0] = g
    rates[:, 1] = g
    c.rates = rates.reshape(-1)
    return c


def config_wing(seed: int = 0, a: float = 400.0, b: float = 250.0, n_layers: int = 8,
                spacing: float = 2.236) -> Tissue:
    """Elliptical wing-disc-like sheet, semi-axes 400 x 250 µm, 8 layers of
    2.5 µm (about 1.0M prisms at 2.236 µm spacing).  Apical layers E = 2000 Pa,
    basal layers 500 Pa.  Radial growth 0.005-0.02/hr plus seeded smooth noise
    of amplitude 0.002/hr.  50 steps of 120 s."""
    rng = np.random.default_rng(seed)
    pos, conn, pl = ellipse_sheet(a, b, spacing, n_layers, 2.5 * n_layers, 0.2 * spacing / 2.236, rng)
    ne = conn.size // 6
    relz = _elem_relative_z(pos, conn)
    E = np.where(relz <= 0.5, 2000.0, 500.0)
    c = Tissue(pos=pos, conn=conn, fixed=_bc_basal_z_fixed(pl),
               ext_visc=_ext_visc_surfaces(pl, 10.0, 10.0), node_placement=pl,
               E=E, nu=np.full(ne, 0.3), eta=np.zeros(ne), rates=np.zeros(3 * ne),
               dt=120.0, n_steps=50, name=f"wing-{ne}")
    cxy = c.centroids()[:, :2]
    rr = np.sqrt((cxy[:, 0] / a) ** 2 + (cxy[:, 1] / b) ** 2)
    base = 0.02 - 0.015 * np.clip(rr, 0.0, 1.0)
    # smooth seeded noise: a few random Fourier modes
    noise = np.zeros(ne)
    for _ in range(6):
        k = rng.uniform(0.5, 3.0, size=2) * math.pi / np.array([a, b])
        ph = rng.uniform(0, 2 * math.pi, size=2)
        noise += np.sin(k[0] * cxy[:, 0] + ph[0]) * np.sin(k[1] * cxy[:, 1] + ph[1])
    noise *= 0.002 / max(1e-12, np.abs(noise).max())
    g = (base + noise) / HOUR
    rates = np.zeros((ne, 3))
    rates[:, 0] = g
    rates[:, 1] = g
    c.rates = rates.reshape(-1)
    return c


def config_tiny(seed: int = 0, n: int = 4, n_layers: int = 2, eta: float = 0.0,
                E: float = 1000.0, nu: float = 0.3, jitter: float = 0.5, spacing: float = 5.0) -> Tissue:
    """Small rectangular sheet used by unit tests (n x n node grid)."""
    rng = np.random.default_rng(seed)
    pos, conn, pl = rect_sheet(n, n, spacing, n_layers, spacing * n_layers, jitter, rng)
    ne = conn.size // 6
    relz = _elem_relative_z(pos, conn)
    r = np.full(ne, 0.01 / HOUR) + np.where(relz <= 0.5, 0.005 / HOUR, 0.0)
    rates = np.zeros((ne, 3))
    rates[:, 0] = r
    rates[:, 1] = r
    return Tissue(pos=pos, conn=conn, fixed=_bc_basal_z_fixed(pl),
                  ext_visc=_ext_visc_surfaces(pl, 10.0, 10.0), node_placement=pl,
                  E=np.full(ne, E) * rng.uniform(0.8, 1.2, size=ne), nu=np.full(ne, nu),
                  eta=np.full(ne, eta), rates=rates.reshape(-1), dt=60.0, n_steps=5,
                  name=f"tiny-{ne}")


def config_facing_sheets(seed: int = 0, n: int = 5, n_layers: int = 2, gap: float = 1.2, eta: float = 0.0,
                         E: float = 1000.0, nu: float = 0.3, jitter: float = 0.3, spacing: float = 5.0,
                         offset=(0.0, 0.0), shuffle: bool = True) -> Tissue:
    """Two n x n sheets whose apical surfaces face each other across `gap`
    (µm): the lower one as config_tiny builds it, the upper one mirrored in z
    (its basal surface on top, its prisms re-ordered so their basal triangle
    stays counter-clockwise seen from the apical side) and shifted in xy by
    `offset`.  Both basal surfaces are fixed in z.  Apical nodes of the two
    sheets closer than the packing detection distance are what the
    reference's packing (Simulation::detectPacingNodes) couples.  `shuffle`
    renumbers the nodes by a seeded permutation, so that packing couples
    start from nodes all over the node order (node 0 keeps its place: the
    reference's bounding box never tests node 0 for the maximum)."""
    rng = np.random.default_rng(seed)
    thick = spacing * n_layers
    pa, ca, la = rect_sheet(n, n, spacing, n_layers, thick, jitter, rng)
    pb, cb, lb = rect_sheet(n, n, spacing, n_layers, thick, jitter, rng)
    pb = pb.reshape(-1, 3).copy()
    pb[:, 0] += offset[0]
    pb[:, 1] += offset[1]
    pb[:, 2] = 2.0 * thick + gap - pb[:, 2]
    cb = cb.reshape(-1, 6)[:, [0, 2, 1, 3, 5, 4]] + pa.size // 3
    pos = np.concatenate([pa.reshape(-1, 3), pb]).reshape(-1)
    conn = np.concatenate([ca.reshape(-1, 6), cb]).reshape(-1).astype(np.int32)
    pl = np.concatenate([la, lb]).astype(np.int32)
    nn = pl.size
    if shuffle:
        perm = np.concatenate([[0], 1 + rng.permutation(nn - 1)])  # new id of each old node
        inv = np.argsort(perm)
        pos = pos.reshape(-1, 3)[inv].reshape(-1)
        pl = pl[inv]
        conn = perm[conn].astype(np.int32)
    ne = conn.size // 6
    rates = np.zeros((ne, 3))
    rates[:, 0] = rates[:, 1] = 0.01 / HOUR
    return Tissue(pos=pos, conn=conn, fixed=_bc_basal_z_fixed(pl), ext_visc=_ext_visc_surfaces(pl, 10.0, 10.0),
                  node_placement=pl, E=np.full(ne, E) * rng.uniform(0.8, 1.2, size=ne), nu=np.full(ne, nu),
                  eta=np.full(ne, eta), rates=rates.reshape(-1), dt=60.0, n_steps=3, name=f"facing-{ne}")


def config_batch_instance(seed: int, min_prisms: int = 1000, max_prisms: int = 50000) -> Tissue:
    """One instance of the batched sweep: prism count log-uniform in
    [1k, 50k], 2-4 layers, rectangular or elliptical, seeded E, nu in
    [0.25, 0.45] and a Gaussian growth map.  20 steps of 60 s."""
    rng = np.random.default_rng(seed)
    target = math.exp(rng.uniform(math.log(min_prisms), math.log(max_prisms)))
    n_layers = int(rng.integers(2, 5))
    tris = target / n_layers
    elliptic = bool(rng.integers(0, 2))
    if elliptic:
        # a structured grid of spacing h puts 2 triangles in each h^2 of the
        # ellipse's area pi a b, b = a / 1.3
        a = math.sqrt(tris * 1.3 * 25.0 / (2.0 * math.pi))
        b = a / 1.3
        pos, conn, pl = ellipse_sheet(a, b, 5.0, n_layers, 5.0 * n_layers, 0.5, rng)
    else:
        n = max(3, int(round(math.sqrt(tris / 2.0))) + 1)
        pos, conn, pl = rect_sheet(n, n, 5.0, n_layers, 5.0 * n_layers, 0.5, rng)
    ne = conn.size // 6
    E = float(rng.uniform(500.0, 2000.0))
    nu = float(rng.uniform(0.25, 0.45))
    c = Tissue(pos=pos, conn=conn, fixed=_bc_basal_z_fixed(pl),
               ext_visc=_ext_visc_surfaces(pl, 10.0, 10.0), node_placement=pl,
               E=np.full(ne, E), nu=np.full(ne, nu), eta=np.zeros(ne), rates=np.zeros(3 * ne),
               dt=60.0, n_steps=20, name=f"batch-{seed}-{ne}")
    cxy = c.centroids()[:, :2]
    lo, hi = cxy.min(axis=0), cxy.max(axis=0)
    centre = lo + rng.uniform(0.3, 0.7, size=2) * (hi - lo)
    width = float(rng.uniform(0.15, 0.35) * (hi - lo).max())
    g = _gaussian_bump(cxy, 0.02 / HOUR, centre, width)
    rates = np.zeros((ne, 3))
    rates[:, 0] = g
    rates[:, 1] = g
    c.rates = rates.reshape(-1)
    return c


def perturbed_state(t: Tissue, seed: int = 1, amp: float = 0.05):
    """A deformed state (uk) near the reference positions plus the previous
    state (un), for evaluating residuals and tangents away from equilibrium."""
    rng = np.random.default_rng(seed)
    un = t.pos + rng.uniform(-amp, amp, size=t.pos.shape) * 0.2
    uk = un + rng.uniform(-amp, amp, size=t.pos.shape)
    return uk, un


def swap_nodes(t: Tissue, a: int, b: int) -> Tissue:
    """The same tissue with node ids a and b exchanged: positions, placement,
    boundary conditions and connectivity follow the nodes."""
    perm = np.arange(t.n_nodes)
    perm[a], perm[b] = b, a
    pos = t.pos.reshape(-1, 3)[perm].reshape(-1).copy()
    fixed = t.fixed.reshape(-1, 3)[perm].reshape(-1).copy()
    ev = t.ext_visc.reshape(-1, 3)[perm].reshape(-1).copy()
    return dataclasses.replace(t, pos=pos, conn=perm[t.conn].astype(np.int32), fixed=fixed, ext_visc=ev,
                               node_placement=t.node_placement[perm].copy())


def grid_growth_inputs(seed: int, nx: int = 5, ny: int = 4, scale: float = 1e-4):
    """Seeded rates (nx, ny, 3) in 1/s and xy angles (nx, ny) in degrees for a
    grid-based growth function: anisotropic in-plane rates, some grid points
    nearly isotropic (aspect ratio below 1.1, so their angle is not used) and
    angles over (-200, 200) degrees, so that neighbouring corners are turned
    by about 90 and 180 degrees from each other."""
    rng = np.random.default_rng(seed)
    r = np.empty((nx, ny, 3))
    r[:, :, 0] = rng.uniform(0.2, 1.0, size=(nx, ny)) * scale
    r[:, :, 1] = r[:, :, 0] * rng.choice([0.3, 0.5, 1.02, 2.5], size=(nx, ny))
    r[:, :, 2] = rng.uniform(-0.2, 0.2, size=(nx, ny)) * scale
    ang = rng.uniform(-200.0, 200.0, size=(nx, ny))
    return r, ang


def growth_Fg(t: Tissue, seed: int = 2, amp: float = 0.02) -> np.ndarray:
    """A seeded non-trivial growth tensor per element (near identity)."""
    rng = np.random.default_rng(seed)
    Fg = np.tile(np.eye(3).reshape(1, 9), (t.n_elems, 1))
    Fg = Fg + rng.uniform(-amp, amp, size=Fg.shape)
    return Fg.reshape(-1)
