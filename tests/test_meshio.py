"""The reference's .mesh input format and save-frame format (host side of the
library, no GPU work): reading the reference's own mesh files where the
reference is present, round trips through our writer, the reference's
orientation correction, and the exact record layout of a save frame."""
import os
import re

import numpy as np
import pytest

from tissuefolding_paperversion_gb300 import api, mesh, meshfile

REF_MESH = os.path.join(os.environ.get("TF_REFERENCE_DIR", "/root/reference"),
                        "TissueFolding", "ToolBox", "MeshGeneration", "2DEllipse")


def _ccw(pos, conn):
    """Prism::checkRotationConsistency3D's test: the basal triangle is
    counter-clockwise seen from the apical side (dot(view, normal) <= 0)."""
    p = pos.reshape(-1, 3)
    c = conn.reshape(-1, 6)
    v1 = p[c[:, 1]] - p[c[:, 0]]
    v2 = p[c[:, 2]] - p[c[:, 0]]
    view = p[c[:, 0]] - p[c[:, 3]]
    return np.einsum("ij,ij->i", view, np.cross(v1, v2)) <= 0


@pytest.mark.skipif(not os.path.isdir(REF_MESH), reason="reference mesh files not present")
@pytest.mark.parametrize("name", ["OnePrism.mesh", "SinglePrism.mesh", "TwoPrisms.mesh", "DoublePrism.mesh",
                                  "Ellipse48hr_04.mesh"])
def test_reads_the_reference_mesh_files(name):
    path = os.path.join(REF_MESH, name)
    with open(path) as f:
        tok = f.read().split()
    n = int(tok[0])
    e = int(tok[1 + 6 * n])
    m = api.read_mesh_file(path)
    assert m["pos"].size == 3 * n and m["conn"].size == 6 * e
    # node records as written
    np.testing.assert_array_equal(m["pos"].reshape(-1, 3)[:, 0], [float(tok[1 + 6 * i]) for i in range(n)])
    np.testing.assert_array_equal(m["placement"], [int(tok[4 + 6 * i]) for i in range(n)])
    assert set(np.unique(m["conn"])) <= set(range(n))
    assert _ccw(m["pos"], m["conn"]).all()
    # element records: node ids and reference shapes as written, with the
    # reference's swap (1<->2, 4<->5) where the prism was clockwise
    base = 2 + 6 * n
    for k in range(e):
        rec = tok[base + 25 * k: base + 25 * (k + 1)]
        assert int(rec[0]) == 1
        ids = np.array([int(v) for v in rec[1:7]])
        ref = np.array([float(v) for v in rec[7:25]]).reshape(6, 3)
        got_ids = m["conn"][6 * k:6 * k + 6]
        got_ref = m["ref_pos"][18 * k:18 * k + 18].reshape(6, 3)
        perm = [0, 1, 2, 3, 4, 5] if np.array_equal(got_ids, ids) else [0, 2, 1, 3, 5, 4]
        np.testing.assert_array_equal(got_ids, ids[perm])
        np.testing.assert_array_equal(got_ref, ref[perm])


def test_round_trip_and_orientation_correction(tmp_path):
    t = mesh.config_tiny(seed=3, n=4, n_layers=2)
    conn = t.conn.reshape(-1, 6).copy()
    conn[0] = conn[0][[0, 2, 1, 3, 5, 4]]          # make prism 0 clockwise
    t2 = mesh.Tissue(**{**t.__dict__, "conn": conn.reshape(-1)})
    path = str(tmp_path / "sheet.mesh")
    meshfile.write_mesh_file(path, t2)
    m = api.read_mesh_file(path)
    np.testing.assert_array_equal(m["pos"], t.pos)
    np.testing.assert_array_equal(m["placement"], t.node_placement)
    # the reader restores the counter-clockwise order of prism 0 like the reference does
    np.testing.assert_array_equal(m["conn"], t.conn)
    assert _ccw(m["pos"], m["conn"]).all()
    lt, info = meshfile.load_tissue(path, E=500.0, eta=100.0)
    assert lt.n_elems == t.n_elems and np.all(lt.E == 500.0) and np.all(lt.eta == 100.0)
    np.testing.assert_array_equal(lt.fixed, t.fixed)


def test_bad_mesh_files_are_rejected(tmp_path):
    p = tmp_path / "bad.mesh"
    p.write_text("2\n0 0 0 0 0 0\n1 0 0 0 0 0\n1\n1 0 1 2 3 4 5\n")   # node id out of range
    with pytest.raises(api.TfError):
        api.read_mesh_file(str(p))
    p.write_text("1\n0 0 0 0 0 0\n1\n4 0 0 0 0 0 0\n")                  # not a prism
    with pytest.raises(api.TfError):
        api.read_mesh_file(str(p))
    with pytest.raises(api.TfError):
        api.read_mesh_file(str(tmp_path / "missing.mesh"))


def test_save_frame_layout(tmp_path):
    t = mesh.config_tiny(seed=4, n=3, n_layers=1)
    path = str(tmp_path / "Save_Frame")
    pos2 = t.pos + 0.125
    api.write_frame(path, 60.0, t.pos, t.conn, t.node_placement, append=False)
    api.write_frame(path, 120.0, pos2, t.conn, t.node_placement)
    lines = open(path).read().splitlines()
    n, e = t.n_nodes, t.n_elems
    per = 1 + 1 + n + 1 + e + 1
    assert len(lines) == 2 * per
    for k, (time, p) in enumerate([(60.0, t.pos), (120.0, pos2)]):
        blk = lines[k * per:(k + 1) * per]
        assert blk[0] == "=============== TIME: " + f"{time:10.6g}" + "=" * 51
        assert blk[-1] == "=============== END OF TIME: " + f"{time:10.6g}" + "=" * 44
        assert int(blk[1]) == n and int(blk[2 + n]) == e
        for i in range(n):
            ln = blk[2 + i]
            assert len(ln) == 3 * 20 + 3 * 4
            xyz = [float(ln[20 * d:20 * (d + 1)]) for d in range(3)]
            np.testing.assert_allclose(xyz, p[3 * i:3 * i + 3], rtol=1e-9)
            assert int(ln[60:64]) == t.node_placement[i]
        for q in range(e):
            ln = blk[3 + n + q]
            assert len(ln) == 4 + 4 + 6 * 9 + 18 * 15
            assert int(ln[0:4]) == 1 and int(ln[4:8]) == 0
            ids = [int(ln[8 + 9 * a:17 + 9 * a]) for a in range(6)]
            assert ids == list(t.conn[6 * q:6 * q + 6])
            assert re.fullmatch(r"( *-?[0-9.e+-]+){18}", ln[62:])
