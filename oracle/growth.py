"""Growth functions: numpy restatement of the reference's growth types 1
(uniform), 2 (ring) and 3 (grid-based), for checking the GPU kernels.  TEST
INFRASTRUCTURE ONLY: imported by tests/, never by the library.

Follows, in TissueFolding/TissueFolding/SourceCode/:
  * ShapeBase::CalculateGrowthRotationByF (ShapeBase.cpp:1656-1810), called
    every step while growth functions exist (Simulation.cpp:5872-5876), and
    the rotated increment of growShapeByFg (:1216-1225);
  * Simulation::calculateGrowth (Simulation.cpp:9651-9666) with
    calculateGrowthUniform (:9757-9799) and calculateGrowthRing (:9801-9885):
    ShapeBase::calculateFgFromRates (ShapeBase.cpp:396-421), R diag(exp(r dt))
    R^T with the function's xy rotation, the ring's rates scaled by
    1 - (d - r_in)/(r_out - r_in) with centre, radii and d in single
    precision;
  * GridBasedGrowthFunction (GrowthFunctionTypes.h:266-609): the aspect-ratio
    test of its constructor (:336-349, threshold 1.1) and
    preCalculateAnglesForCompatibleAveraging (:427-579): corner angles brought
    to [0, pi] and next to the first corner that carries one, x/y rates
    swapped where a corner turns by about 90 or 270 degrees;
  * Simulation::calculateTissueHeight (Simulation.cpp:3280-3330) with
    Prism::IsThisNodeMyBasal / getCorrecpondingApical / getElementHeight
    (Prism.cpp:1497-1531);
  * Simulation::calculateBoundingBox (Simulation.cpp:9148-9185), its running
    "else if" included: a node that lowers the minimum is not a candidate for
    the maximum;
  * ShapeBase::setInitialZPosition (ShapeBase.cpp:612-627),
    calculateRelativePosInBoundingBox (:1842-1848) with getCentre (:240-250);
  * ShapeBase::setTissuePlacement (ShapeBase.cpp:705-770),
    Simulation::fillInElementColumnLists (Simulation.cpp:7612-7624) with
    Prism::constructElementStackList (Prism.cpp:2542-2584) and
    Simulation::updateRelativePositionsToApicalPositioning (:5987-6003);
  * ShapeBase::convertRelativePosToGridIndex (ShapeBase.cpp:633-660) and
    calculateFgFromGridCorners (:432-562) for columnar prisms (tissue weight
    1), Simulation::calculateGrowthGridBased (Simulation.cpp:10065-10114),
    ShapeBase::updateGrowthIncrement (:567-586) and growShapeByFg
    (:1215-1251).
"""
from __future__ import annotations

import math

import numpy as np

from tissuefolding_paperversion_gb300 import mesh

BOX_INIT = 100000.0   # calculateBoundingBox's starting corners


def element_placement(conn, node_placement):
    """(E,) 3 lateral, 1 apical, 0 basal, 2 mid-line or spanning."""
    c = np.asarray(conn).reshape(-1, 6)
    p = np.asarray(node_placement)[c]
    ap = (p == 1).any(axis=1)
    ba = (p == 0).any(axis=1)
    la = (p == 3).any(axis=1)
    out = np.full(c.shape[0], 2, dtype=np.int32)
    out[ba & ~ap] = 0
    out[ap & ~ba] = 1
    out[la] = 3
    return out


def bounding_box(pos):
    """(lo (3,), size (3,)) as calculateBoundingBox computes them."""
    p = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
    lo = np.minimum(BOX_INIT, p.min(axis=0)) if len(p) else np.full(3, BOX_INIT)
    hi = np.full(3, -BOX_INIT)
    for k in range(3):
        x = p[:, k]
        before = np.minimum.accumulate(np.concatenate([[BOX_INIT], x[:-1]]))
        before = np.minimum(before, BOX_INIT)
        cand = x[~(x < before)]
        if cand.size:
            hi[k] = max(-BOX_INIT, cand.max())
    return lo, hi - lo


def centres(pos, conn):
    """Prism centres, summed node by node in connectivity order, then / 6."""
    p = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
    c = np.asarray(conn).reshape(-1, 6)
    s = np.zeros((c.shape[0], 3))
    for a in range(6):
        s = s + p[c[:, a]]
    return s / 6


def tissue_height(pos, conn, node_placement):
    """(layers, height) from the first basal node up its column."""
    p = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
    c = np.asarray(conn).reshape(-1, 6)
    pl = np.asarray(node_placement)
    basal = np.nonzero(pl == 0)[0]
    if basal.size == 0:
        return 0, 0.0
    cur = int(basal[0])
    layers, height = 0, 0.0
    for _ in range(c.shape[0] + 1):
        if pl[cur] == 1:
            break
        hit = np.nonzero((c[:, :3] == cur).any(axis=1))[0]
        if hit.size == 0:
            break
        e = int(hit[0])
        d = p[c[e, 0]] - p[c[e, 3]]
        height += math.pow(float(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]), 0.5)
        layers += 1
        cur = int(c[e, 3 + int(np.nonzero(c[e, :3] == cur)[0][0])])
    return layers, height


def columns(conn, node_placement, layers):
    """(E,) the prism whose bounding-box position each prism takes."""
    c = np.asarray(conn).reshape(-1, 6)
    ne = c.shape[0]
    place = element_placement(c, node_placement)
    by_basal = {}
    for e in range(ne):
        by_basal.setdefault(tuple(sorted(c[e, :3])), e)
    src = np.arange(ne)
    if layers < 3:
        return src
    for e in np.nonzero(place == 0)[0]:
        col = [int(e)]
        for _ in range(1, layers):
            nxt = by_basal.get(tuple(sorted(c[col[-1], 3:])))
            if nxt is None or nxt == col[-1]:
                break
            col.append(nxt)
        if len(col) != layers or place[col[-1]] != 1:
            continue
        for i in range(layers - 2):
            src[col[i]] = col[-1]
    return src


def relative_positions(pos, conn, src):
    """(E, 2) positions in the bounding box after the column rule."""
    lo, size = bounding_box(pos)
    cen = centres(pos, conn)
    rel = np.stack([(cen[:, 0] - lo[0]) / size[0], (cen[:, 1] - lo[1]) / size[1]], axis=1)
    return rel[src]


def initial_state(pos0, conn, node_placement):
    """Tissue height, initial relative z, columns and pinned positions."""
    layers, height = tissue_height(pos0, conn, node_placement)
    lo, _ = bounding_box(pos0)
    cz = centres(pos0, conn)[:, 2]
    relz = np.clip(1.0 - (cz - lo[2]) / height, 0.0, 1.0)
    src = columns(conn, node_placement, layers)
    return {"layers": layers, "height": height, "relz": relz, "src": src,
            "rel0": relative_positions(pos0, conn, src)}


def compatible_corners(rates, angles_deg=None):
    """rates (nx, ny, 3), angles (nx, ny) degrees -> per cell (nx-1, ny-1):
    corner rates (4, 3), corner angles (4,), corners without an angle (4,)."""
    r = np.asarray(rates, dtype=np.float64)
    nx, ny = r.shape[:2]
    ang = np.zeros((nx, ny)) if angles_deg is None else np.asarray(angles_deg, dtype=np.float64) * math.pi / 180.0
    cg = np.zeros((nx - 1, ny - 1, 4, 3))
    ca = np.zeros((nx - 1, ny - 1, 4))
    ce = np.zeros((nx - 1, ny - 1, 4), dtype=bool)

    def over(i, j):
        ar = r[i, j, 0] / r[i, j, 1]
        if ar < 0:
            ar *= -1.0
        if ar < 1.0:
            ar = 1 / ar
        return not ar < 1.1

    pi = math.pi
    for ix in range(nx - 1):
        for iy in range(ny - 1):
            pts = [(ix, iy), (ix + 1, iy), (ix, iy + 1), (ix + 1, iy + 1)]
            g = [list(r[i, j]) for i, j in pts]
            a = [0.0] * 4
            el = [False] * 4
            for c, (i, j) in enumerate(pts):
                if over(i, j):
                    a[c] = float(ang[i, j])
                else:
                    el[c] = True
            for c in range(4):
                while a[c] < 0:
                    a[c] += pi
                while a[c] > pi:
                    a[c] -= pi
            base, tet = 3, 0.0
            for c in range(4):
                if not el[c]:
                    base, tet = c, a[c]
                    break
            flip = [False] * 4
            for c in range(base, 4):
                d = a[c] - tet
                if d > 0:
                    if pi / 4.0 <= d < 3.0 * pi / 4.0:
                        a[c], flip[c] = a[c] - pi / 2.0, True
                    elif 3.0 * pi / 4.0 <= d < 5.0 * pi / 4.0:
                        a[c] = a[c] - pi
                    elif 5.0 * pi / 4.0 <= d < 7.0 * pi / 4.0:
                        a[c], flip[c] = a[c] - 6.0 * pi / 4.0, True
                    elif d >= 7.0 * pi / 4.0:
                        a[c] = a[c] - 2.0 * pi
                elif d < 0:
                    if -3.0 * pi / 4.0 < d <= -pi / 4.0:
                        a[c], flip[c] = a[c] + pi / 2.0, True
                    elif -5.0 * pi / 4.0 < d <= -3.0 * pi / 4.0:
                        a[c] = a[c] + pi
                    elif -7.0 * pi / 4.0 < d <= -5.0 * pi / 4.0:
                        a[c], flip[c] = a[c] + 6.0 * pi / 4.0, True
                    elif d <= -7.0 * pi / 4.0:
                        a[c] = a[c] + 2.0 * pi
            for c in range(4):
                if flip[c]:
                    g[c][0], g[c][1] = g[c][1], g[c][0]
            cg[ix, iy] = g
            ca[ix, iy] = a
            ce[ix, iy] = el
    return cg, ca, ce


def grid_index(rel, nx, ny):
    """convertRelativePosToGridIndex: (ix, iy, fx, fy) per prism."""
    rx = rel[:, 0] * float(np.float32(nx - 1))
    ry = rel[:, 1] * float(np.float32(ny - 1))
    ix = np.floor(rx).astype(np.int64)
    iy = np.floor(ry).astype(np.int64)
    fx = rx - ix
    fy = ry - iy
    hi = ix >= nx - 1
    lo = ~hi & (ix < 0)
    ix = np.where(hi, nx - 2, np.where(lo, 0, ix))
    fx = np.where(hi, 1.0, np.where(lo, 0.0, fx))
    hi = iy >= ny - 1
    lo = ~hi & (iy < 0)
    iy = np.where(hi, ny - 2, np.where(lo, 0, iy))
    fy = np.where(hi, 1.0, np.where(lo, 0.0, fy))
    return ix, iy, fx, fy


def dgemm3(A, B, trans_b=False):
    """Stacked 3x3 products C = A B (or A B^T) summed over k from 0 as the
    reference's gsl_blas_dgemm stand-in does: ((0 + a0 b0) + a1 b1) + a2 b2."""
    Bt = np.transpose(B, (0, 2, 1)) if trans_b else B
    C = np.zeros(np.broadcast_shapes(A.shape, Bt.shape))
    for i in range(3):
        for j in range(3):
            acc = np.zeros(C.shape[0])
            for k in range(3):
                acc = acc + A[:, i, k] * Bt[:, k, j]
            C[:, i, j] = acc
    return C


def grid_increments(rel, relz, corners, dt, interp=1, zmin=0.0, zmax=1.0):
    """(E, 3, 3) growth increments of one grid function
    (calculateFgFromGridCorners, operations in the reference's order)."""
    cg, ca, ce = corners
    nx, ny = cg.shape[0] + 1, cg.shape[1] + 1
    ne = rel.shape[0]
    ix, iy, fx, fy = grid_index(rel, nx, ny)
    g = cg[ix, iy]          # (E, 4, 3)
    an = ca[ix, iy]         # (E, 4)
    el = ce[ix, iy]         # (E, 4)
    ux, uy = 1.0 - fx, 1.0 - fy
    if interp == 0:
        corner = np.where(fx > 0.5, np.where(fy > 0.5, 3, 1), np.where(fy > 0.5, 2, 0))
        growth = g[np.arange(ne), corner]
        angle = np.zeros(ne)
    else:
        fe = np.zeros(ne)
        for c, w in enumerate((ux * uy, fx * uy, ux * fy, fx * fy)):
            fe = np.where(el[:, c], fe + w, fe)
        angle = an[:, 0] * ux * uy + an[:, 1] * fx * uy + an[:, 2] * ux * fy + an[:, 3] * fx * fy
        safe = np.where(fe < 1.0, 1.0 - fe, 1.0)
        angle = np.where(fe > 0, np.where(fe >= 0.9999999, 0.0, angle / safe), angle)
        growth = (g[:, 0] * ux[:, None] * uy[:, None] + g[:, 1] * fx[:, None] * uy[:, None]
                  + g[:, 2] * ux[:, None] * fy[:, None] + g[:, 3] * fx[:, None] * fy[:, None])
    inc = np.zeros((ne, 3, 3))
    for k in range(3):
        inc[:, k, k] = np.exp(growth[:, k] * dt)
    rot = angle != 0.0
    if rot.any():
        c, s = np.cos(angle[rot]), np.sin(angle[rot])
        R = np.zeros((int(rot.sum()), 3, 3))
        R[:, 0, 0], R[:, 0, 1], R[:, 1, 0], R[:, 1, 1], R[:, 2, 2] = c, -1.0 * s, s, c, 1.0
        inc[rot] = dgemm3(dgemm3(R, inc[rot]), R, trans_b=True)
    off = (relz < zmin) | (relz > zmax)
    inc[off] = np.eye(3)
    return inc


def rotation(angle):
    c, s = math.cos(angle), math.sin(angle)
    return np.array([[c, -1.0 * s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])


def rates_increment(r, R, dt):
    """calculateFgFromRates, tissue weight 1: r (E, 3) -> (E, 3, 3)."""
    ne = r.shape[0]
    d = np.zeros((ne, 3, 3))
    for k in range(3):
        d[:, k, k] = np.exp(r[:, k] * 1.0 * dt)
    Rs = np.broadcast_to(R, (ne, 3, 3))
    return dgemm3(dgemm3(Rs, d), Rs, trans_b=True)


def ring_scale(pos, conn, fn):
    """(E,) the ring's rate scale per prism, NaN outside the ring."""
    cen = centres(pos, conn)
    f32 = np.float32
    cx, cy, rin, rout = f32(fn["cx"]), f32(fn["cy"]), f32(fn["rin"]), f32(fn["rout"])
    dx = float(cx) - cen[:, 0]
    dy = float(cy) - cen[:, 1]
    d2 = dx * dx + dy * dy
    rin2, rout2 = float(rin * rin), float(rout * rout)
    inside = (d2 > rin2) & (d2 < rout2)
    dist = np.sqrt(d2).astype(np.float32)
    frac = ((dist - rin) / (rout - rin)).astype(np.float32)
    return np.where(inside, 1.0 - frac.astype(np.float64), np.nan)


def shape_derivatives():
    """(6, 3, 6) derivatives of the prism's shape functions at its 6 Gauss
    points with respect to the parametric coordinates
    (Prism::setShapeFunctionDerivatives, Prism.cpp:655-680; Gauss points of
    the Prism constructor, :123-148)."""
    s = 1.0 / math.pow(3, 0.5)
    pts = [(1 / 6, 1 / 6, s), (2 / 3, 1 / 6, s), (1 / 6, 2 / 3, s), (1 / 6, 1 / 6, -s), (2 / 3, 1 / 6, -s),
           (1 / 6, 2 / 3, -s)]
    out = np.zeros((6, 3, 6))
    for p, (eta, nu, zeta) in enumerate(pts):
        al, be, lam = (1 - zeta) / 2, (1 + zeta) / 2, 1 - eta - nu
        out[p] = [[-al, al, 0, -be, be, 0], [-al, 0, al, -be, 0, be],
                  [-lam / 2, -eta / 2, -nu / 2, lam / 2, eta / 2, nu / 2]]
    return out


def growth_rotations(pos, conn, inv_dXde):
    """ShapeBase::CalculateGrowthRotationByF per prism: (rotated (E,), Rz (E, 3, 3)).
    The Gauss-weighted deformation gradient of the current shape
    (calculateTriPointFForRatation, ShapeBase.cpp:1674-1687, with
    Prism::calculateCurrTriPointFForRotation, Prism.cpp:730-744), its rotation
    U V^T from the singular value decomposition (calculate3DRotMatFromF,
    ShapeBase.cpp:1731-1810: rotated if an off-diagonal entry exceeds 0.017),
    and the angle about z (disassembleRotationMatrixForZ, :1690-1721)."""
    x = np.asarray(pos, dtype=np.float64).reshape(-1, 3)[np.asarray(conn).reshape(-1, 6)]
    dN = shape_derivatives()
    F = np.zeros((x.shape[0], 3, 3))
    for gp in range(6):
        Jt = np.einsum("ra,eac->erc", dN[gp], x)
        Fgp = np.transpose(Jt, (0, 2, 1)) @ inv_dXde[:, gp]
        F = F + Fgp * (1.0 / 6.0)
    U, _, Vt = np.linalg.svd(F)
    R = U @ Vt
    off = np.abs(R - np.eye(3) * np.diagonal(R, axis1=1, axis2=2)[:, :, None]).max(axis=(1, 2)) > 0.017
    tz = np.arctan2(R[:, 0, 1], R[:, 0, 0])
    rot = off & (np.abs(tz) > 0.017)
    c, s = np.cos(tz), np.sin(tz)
    Rz = np.zeros((x.shape[0], 3, 3))
    Rz[:, 0, 0], Rz[:, 0, 1], Rz[:, 1, 0], Rz[:, 1, 1], Rz[:, 2, 2] = c, -1.0 * s, s, c, 1.0
    return rot, Rz


class GrowthOracle:
    """Growth functions on one tissue: the state the reference keeps for them."""

    def __init__(self, pos0, conn, node_placement, ref_pos=None):
        self.conn = np.asarray(conn).reshape(-1, 6)
        self.state = initial_state(pos0, self.conn, node_placement)
        self.fns = []
        self.interp = 1
        self.pinned = False
        X = (np.asarray(pos0, dtype=np.float64).reshape(-1, 3)[self.conn] if ref_pos is None
             else np.asarray(ref_pos, dtype=np.float64).reshape(-1, 6, 3))
        dN = shape_derivatives()
        self.inv_dXde = np.stack([np.linalg.inv(np.transpose(np.einsum("ra,eac->erc", dN[gp], X), (0, 2, 1)))
                                  for gp in range(6)], axis=1)

    @staticmethod
    def _window(init_time, end_time, zmin, zmax):
        return {"t0": float(np.float32(init_time)), "t1": float(np.float32(end_time)), "zmin": zmin, "zmax": zmax}

    def add_grid_growth(self, rates, angles_deg=None, init_time=-1e30, end_time=1e30, zmin=0.0, zmax=1.0):
        """A grid-based function (type 3)."""
        self.fns.append({"type": 3, "corners": compatible_corners(rates, angles_deg),
                         **self._window(init_time, end_time, zmin, zmax)})

    add = add_grid_growth

    def add_uniform_growth(self, rates, angle_rad=0.0, init_time=-1e30, end_time=1e30, zmin=0.0, zmax=1.0):
        self.fns.append({"type": 1, "rate": np.asarray(rates, dtype=np.float64), "R": rotation(angle_rad),
                         **self._window(init_time, end_time, zmin, zmax)})

    def add_ring_growth(self, centre, inner_radius, outer_radius, rates, angle_rad=0.0, init_time=-1e30, end_time=1e30,
                 zmin=0.0, zmax=1.0):
        self.fns.append({"type": 2, "rate": np.asarray(rates, dtype=np.float64), "R": rotation(angle_rad),
                         "cx": centre[0], "cy": centre[1], "rin": inner_radius, "rout": outer_radius,
                         **self._window(init_time, end_time, zmin, zmax)})

    def repin(self, pos):
        self.state["rel0"] = relative_positions(pos, self.conn, self.state["src"])

    def increment(self, pos, time, dt, rates=None):
        """The step's growth increment (E, 3, 3): the per-element rates'
        diag(exp(rate dt)), then each active function's increment multiplied
        on the left (updateGrowthIncrement)."""
        ne = self.conn.shape[0]
        total = np.broadcast_to(np.eye(3), (ne, 3, 3)).copy()
        if rates is not None:
            r = np.asarray(rates, dtype=np.float64).reshape(-1, 3)
            for k in range(3):
                total[:, k, k] = np.exp(r[:, k] * 1.0 * dt)
        if not self.fns:
            return total
        active = [f for f in self.fns if f["t0"] <= time < f["t1"]]
        rel = self.state["rel0"] if self.pinned else relative_positions(pos, self.conn, self.state["src"])
        relz = self.state["relz"]
        for f in active:
            if f["type"] == 3:
                inc = grid_increments(rel, relz, f["corners"], dt, self.interp, f["zmin"], f["zmax"])
            else:
                r = np.broadcast_to(f["rate"], (ne, 3)).copy()
                keep = (relz >= f["zmin"]) & (relz <= f["zmax"])
                if f["type"] == 2:
                    sf = ring_scale(pos, self.conn, f)
                    keep &= ~np.isnan(sf)
                    r = r * np.where(np.isnan(sf), 0.0, sf)[:, None]
                inc = rates_increment(r, f["R"], dt)
                inc[~keep] = np.eye(3)
            total = dgemm3(inc, total)
        # growShapeByFg with rotatedGrowth (ShapeBase.cpp:1216-1225): Rz G Rz^T
        rot, Rz = growth_rotations(pos, self.conn, self.inv_dXde)
        if rot.any():
            total[rot] = dgemm3(dgemm3(Rz[rot], total[rot]), Rz[rot], trans_b=True)
        return total

    def grow(self, Fg, pos, time, dt, rates=None):
        """Fg (E, 3, 3) after one step's growth (growShapeByFg)."""
        Fg = np.broadcast_to(np.asarray(Fg, dtype=np.float64), (self.conn.shape[0], 3, 3))
        return dgemm3(self.increment(pos, time, dt, rates), Fg)


FIXTURES = ["steps_grid_growth", "steps_grid_growth_pinned"]
MIXED_FIXTURE = "steps_growth_functions"
ROTATED_FIXTURE = "steps_growth_rotated"


def add_functions(obj, fns):
    """Adds function descriptors ({"kind": "uniform" | "ring" | "grid", ...
    arguments}) to a solver, the reference driver or a GrowthOracle -- all
    three name the calls add_uniform_growth / add_ring_growth /
    add_grid_growth."""
    for f in fns:
        kw = {k: v for k, v in f.items() if k != "kind"}
        getattr(obj, "add_" + f.get("kind", "grid") + "_growth")(**kw)


def mixed_case():
    """Tissue and functions of the steps_growth_functions fixture: a 3-layer
    sheet with a uniform function turned by 0.7 rad in the apical 60 %, a
    ring, a grid function, and a second ring from t = 60 s in the basal 70 %,
    applied in this order after the per-element rates."""
    t = mesh.config_tiny(seed=23, n=7, n_layers=3, eta=20.0)
    ra, aa = mesh.grid_growth_inputs(34, 4, 4)
    fns = [dict(kind="uniform", rates=[3e-5, 1e-5, -2e-6], angle_rad=0.7, zmin=0.0, zmax=0.6),
           dict(kind="ring", centre=(14.3, 12.1), inner_radius=4.0, outer_radius=19.0, rates=[5e-5, 2e-5, 0.0],
                angle_rad=-0.4),
           dict(kind="grid", rates=ra, angles_deg=aa),
           dict(kind="ring", centre=(2.0, 30.0), inner_radius=0.0, outer_radius=25.0, rates=[1e-5, 4e-5, 1e-6],
                init_time=60.0, zmin=0.3, zmax=1.0)]
    return t, fns


def fixture_case(name):
    """Tissue, grid functions, interpolation and pinning of a grid growth
    fixture (tests/golden/make_golden.py --only-grid).  steps_grid_growth: a
    4-layer sheet renumbered so that node 0 alone holds the largest x (the
    reference's bounding box then misses the true maximum), two functions,
    the second only in the basal half and from t = 60 s, bilinear, current
    positions.  steps_grid_growth_pinned: a 3-layer sheet, one function,
    nearest grid point, positions pinned on the initial mesh."""
    if name == "steps_grid_growth":
        t = mesh.config_tiny(seed=21, n=6, n_layers=4, eta=50.0)
        t = mesh.swap_nodes(t, 0, int(np.argmax(t.pos.reshape(-1, 3)[:, 0])))
        t.pos[0] += 0.4
        ra, aa = mesh.grid_growth_inputs(31, 5, 4)
        rb, ab = mesh.grid_growth_inputs(32, 3, 3, scale=5e-5)
        fns = [dict(rates=ra, angles_deg=aa, init_time=-1e30, end_time=1e30, zmin=0.0, zmax=1.0),
               dict(rates=rb, angles_deg=ab, init_time=60.0, end_time=1e30, zmin=0.5, zmax=1.0)]
        return t, fns, 1, False
    if name == "steps_grid_growth_pinned":
        t = mesh.config_tiny(seed=22, n=5, n_layers=3, eta=0.0)
        ra, aa = mesh.grid_growth_inputs(33, 4, 4)
        return t, [dict(rates=ra, angles_deg=aa, init_time=-1e30, end_time=1e30, zmin=0.0, zmax=1.0)], 0, True
    raise KeyError(name)


GridGrowthOracle = GrowthOracle


def turned(pos, degrees):
    """Positions turned by `degrees` about the z axis."""
    a = math.radians(degrees)
    p = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
    q = p.copy()
    q[:, 0] = math.cos(a) * p[:, 0] - math.sin(a) * p[:, 1]
    q[:, 1] = math.sin(a) * p[:, 0] + math.cos(a) * p[:, 1]
    return q.reshape(-1)


def rotated_case():
    """Tissue, start positions and functions of the steps_growth_rotated
    fixture: a 2-layer sheet whose start shape is its mesh turned by 20
    degrees about z (a rigid turn: no strain), an anisotropic uniform function
    and a grid function; every prism's growth increment is turned with it."""
    t = mesh.config_tiny(seed=24, n=6, n_layers=2, eta=30.0)
    ra, aa = mesh.grid_growth_inputs(35, 4, 5)
    fns = [dict(kind="uniform", rates=[5e-5, 1e-5, 0.0], angle_rad=0.2), dict(kind="grid", rates=ra, angles_deg=aa)]
    return t, turned(t.pos, 20.0), fns


def stretched(pos, eps, centre=None):
    """Positions stretched in x and y by 1 + eps about `centre` (a pure
    stretch: the rotation of every prism's deformation gradient is I)."""
    p = np.asarray(pos, dtype=np.float64).reshape(-1, 3).copy()
    c = p.mean(axis=0) if centre is None else np.asarray(centre, dtype=np.float64)
    p[:, :2] = c[:2] + (1.0 + eps) * (p[:, :2] - c[:2])
    return p.reshape(-1)


# Start shapes at the turn's thresholds: (label, kind, value, turned).  A rigid
# turn by phi gives F = Rz(phi), whose distance 2|F - I| (Frobenius) crosses
# 0.017 at phi = 0.00601 and whose off-diagonal entries (sin phi) and angle
# cross the reference's 0.017 at phi = 0.0170; a stretch by 1 + eps in x and y
# has 2|F - I| = 2 sqrt(2) eps (0.017 at eps = 0.00601) and no rotation.
TURN_THRESHOLD_CASES = [
    ("turn below the distance bound", "turn", 0.0059, False),
    ("turn above the distance bound", "turn", 0.0061, False),
    ("turn just below 0.017", "turn", 0.0169, False),
    ("turn just above 0.017", "turn", 0.0171, True),
    ("turn back just above 0.017", "turn", -0.0171, True),
    ("stretch below the distance bound", "stretch", 0.0059, False),
    ("stretch above the distance bound", "stretch", 0.0061, False),
]


def threshold_start(t, kind, value):
    """Start positions of one TURN_THRESHOLD_CASES entry for tissue t."""
    if kind == "turn":
        return turned(t.pos, math.degrees(value))
    return stretched(t.pos, value)
