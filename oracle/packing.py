"""Packing between tissue surfaces: numpy restatement of the reference's
implicit packing, for checking the GPU kernels.  TEST INFRASTRUCTURE ONLY:
imported by tests/, never by the library.

Follows, in TissueFolding/TissueFolding/SourceCode/:
  * Prism::calculateReferenceVolume (Prism.cpp:876-908) with
    ShapeBase::calculateVolumeForInputShapeStructure (ShapeBase.cpp:3362-3395):
    the reference volume of a prism from 8 triangles and its centre;
  * ShapeBase::growShapeByFg (ShapeBase.cpp:1243-1245): the volume per node
    det(Fg) * V_ref / 6, and Simulation::updateNodeMasses
    (Simulation.cpp:7552-7561): node mass = sum of the volumes per node of
    its prisms, in prism order;
  * Simulation::getAverageSideLength (Simulation.cpp:3205-3265): the mean
    apical (and, for prisms with a basal node, basal) side length, and the
    detection grid, whose only populated cell is [0][0] (prism centres lie
    inside the bounding box, at fractions in [0, 1));
  * Simulation::calculateBoundingBox (Simulation.cpp:9148-9185), with its
    running "else if" (oracle/growth.py bounding_box);
  * Simulation::detectPacingNodes (Simulation.cpp:8167-8440): couples of
    packing-eligible nodes (Node::checkIfNodeHasPacking, Node.cpp:133-150:
    mass > 0, apical or basal) on the same surface, not neighbours, closer
    than 0.4 x the grid value of the first node's cell; weights = unit vector
    from the second node to the first; the merge loop (:8426) drops the
    couples found from the last of 16 node segments;
  * Simulation::calculatePackingForcesImplicit3D (:7149-7203),
    calculatePackingJacobian3D (:7205-7300), addPackingForces (:8869-8900).
"""
from __future__ import annotations

import numpy as np

from oracle.growth import bounding_box

MULTIPLIER = 5000.0      # packingMultiplier (Simulation.cpp:8187)
SATURATION = 5.0         # sigmoidSaturationForPacking (:8188)
FACES = [(0, 1, 2), (3, 4, 5), (0, 1, 3), (1, 3, 4), (1, 2, 4), (2, 4, 5), (0, 2, 3), (2, 3, 5)]


def reference_volumes(ref):
    """ref: (E, 6, 3) reference prism shapes -> (E,) volumes."""
    ref = np.asarray(ref, dtype=np.float64)
    centre = ref.sum(axis=1) / 6.0
    vol = np.zeros(ref.shape[0])
    for f in FACES:
        p0, p1, p2 = ref[:, f[0]], ref[:, f[1]], ref[:, f[2]]
        v1, v2, vm = p1 - p0, p2 - p0, centre - p0
        b = np.stack([v1[:, 1] * v2[:, 2] - v1[:, 2] * v2[:, 1],
                      v1[:, 2] * v2[:, 0] - v1[:, 0] * v2[:, 2],
                      v1[:, 0] * v2[:, 1] - v1[:, 1] * v2[:, 0]], axis=1)
        nb = np.sqrt(b[:, 0] * b[:, 0] + b[:, 1] * b[:, 1] + b[:, 2] * b[:, 2])
        area = nb / 2
        h = np.abs((vm[:, 0] * b[:, 0] + vm[:, 1] * b[:, 1] + vm[:, 2] * b[:, 2]) / nb)
        vol += 1.0 / 3.0 * (h * area)
    return vol


def det3(Fg):
    """ShapeBase::determinant3by3Matrix (ShapeBase.cpp:2050-2056); Fg (E, 3, 3)."""
    F = np.asarray(Fg, dtype=np.float64)
    d = F[:, 0, 0] * (F[:, 1, 1] * F[:, 2, 2] - F[:, 1, 2] * F[:, 2, 1])
    d = d - F[:, 0, 1] * (F[:, 1, 0] * F[:, 2, 2] - F[:, 1, 2] * F[:, 2, 0])
    d = d + F[:, 0, 2] * (F[:, 1, 0] * F[:, 2, 1] - F[:, 1, 1] * F[:, 2, 0])
    return d


def node_masses(conn, n_nodes, vref, Fg):
    """Masses in prism order (updateNodeMasses)."""
    per = det3(np.asarray(Fg).reshape(-1, 3, 3)) * vref / 6
    m = np.zeros(n_nodes)
    c = np.asarray(conn).reshape(-1, 6)
    for e in range(c.shape[0]):
        for a in range(6):
            m[c[e, a]] += per[e]
    return m


def _side_avg(P, c, pairs):
    """Prism::getApicalSideLengthAverage / getBasalSideLengthAverage
    (Prism.cpp:1443-1490) for every prism: mean of the non-zero side lengths
    of the triangle (0 if all are zero)."""
    s = np.zeros(c.shape[0])
    n = np.zeros(c.shape[0])
    for a, b in pairs:
        d = P[c[:, a]] - P[c[:, b]]
        d2 = d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2]
        pos = d2 > 0
        s = np.where(pos, s + np.sqrt(d2), s)
        n = n + pos
    return np.where(n > 0, s / np.maximum(n, 1), s)


def side_lengths(pos, conn, placement):
    """(colAverageSideLength, grid[0][0]) of getAverageSideLength for a
    tissue of columnar prisms (sums in prism order)."""
    P = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
    c = np.asarray(conn).reshape(-1, 6)
    pl = np.asarray(placement)
    ap = _side_avg(P, c, [(3, 4), (3, 5), (4, 5)])
    bs = _side_avg(P, c, [(0, 1), (0, 2), (1, 2)])
    basal = np.any(pl[c] == 0, axis=1)            # basal placement or spans the whole tissue
    dsum, n, gsum = 0.0, 0, 0.0
    for e in range(c.shape[0]):
        v = ap[e]
        if v > 0:
            dsum += v
            n += 1
        if basal[e]:
            v = bs[e]
            if v > 0:
                dsum += v
                n += 1
        gsum += v
    return dsum / n, gsum / c.shape[0]


def neighbours(conn, n_nodes):
    """Node::immediateNeigs as sets (ShapeBase::fillNodeNeighbourhood)."""
    nb = [set() for _ in range(n_nodes)]
    for row in np.asarray(conn).reshape(-1, 6):
        for a in row:
            nb[a].update(int(b) for b in row if b != a)
    return nb


def detect(pos, conn, placement, masses, drop_last_segment=True, masters=None, nb=None):
    """Couples of detectPacingNodes at positions `pos`: dict with nodes
    (n, 2), w (n, 3), mbar (n,), threshold, detect.  `masters` restricts the
    scan to those first nodes (a timing sample); `nb` passes precomputed
    neighbour sets."""
    P = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
    nn = P.shape[0]
    pl = np.asarray(placement)
    col, g00 = side_lengths(pos, conn, placement)
    r = 0.4 * g00
    t2_00 = r * r
    bb0, bbs = bounding_box(P)
    eligible = (masses != 0) & ((pl == 0) | (pl == 1))
    if nb is None:
        nb = neighbours(conn, nn)
    seg = max(nn // 16, 1)
    last = (nn // seg - 1) * seg
    c0, c1, w = [], [], []
    for a in (range(nn) if masters is None else masters):
        if not eligible[a] or (drop_last_segment and a >= last):
            continue
        gx = np.floor((P[a, 0] - bb0[0]) / bbs[0])
        gy = np.floor((P[a, 1] - bb0[1]) / bbs[1])
        t2 = t2_00 if (gx == 0 and gy == 0) else 0.0
        if t2 <= 0:
            continue
        b = np.arange(a + 1, nn)
        d = P[a] - P[b]
        d2 = d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2]
        ok = eligible[b] & (pl[b] == pl[a]) & (d2 < t2)
        for k in np.flatnonzero(ok):           # partners in node order
            if int(b[k]) in nb[a]:
                continue
            c0.append(a)
            c1.append(int(b[k]))
            w.append(d[k] / d2[k] ** 0.5)
    nodes = np.array([c0, c1], dtype=np.int64).T.reshape(-1, 2)
    w = np.array(w, dtype=np.float64).reshape(-1, 3)
    mbar = 0.5 * (masses[nodes[:, 0]] + masses[nodes[:, 1]]) if len(nodes) else np.zeros(0)
    return {"nodes": nodes, "w": w, "mbar": mbar, "threshold": 0.4 * col, "detect": r}


def forces_and_jacobian(pos, pk):
    """Packing forces (3N, added to g) and the Jacobian entries at positions
    `pos`: a list of (row, col, value) K increments in the reference's order.
    Fixed DOFs are left to calcutateFixedK (the caller masks them)."""
    P = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
    f = np.zeros(P.size)
    trip = []
    k = SATURATION / pk["threshold"]
    for i, (a, b) in enumerate(pk["nodes"]):
        m = pk["mbar"][i]
        for d in range(3):
            wd = pk["w"][i, d]
            dd = P[a, d] - P[b, d]
            if wd > 0:
                dd = -dd
            F = MULTIPLIER * m / (1 + np.exp(k * (-1.0 * dd))) * wd
            f[3 * a + d] += F
            f[3 * b + d] -= F
            sig = 1 / (1 + np.exp(k * (-1.0 * dd)))
            d0 = sig * (1 - sig) * MULTIPLIER * m * wd * k
            d1 = -1.0 * d0
            if wd > 0:
                d0, d1 = -d0, -d1
            ra, rb = 3 * a + d, 3 * b + d
            trip += [(ra, ra, -d0), (ra, rb, -d1), (rb, rb, -d0), (rb, ra, -d1)]
    return f, trip
