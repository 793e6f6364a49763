""".cdb input in the library (nla3d_gb300.cdb, following readCdbFile,
FEReaders.cpp:321-729, and compressNumbers, FEReaders.cpp:35-80).

* A file written here from a generated hex block, in both EBLOCK layouts,
  with sparse node numbers, CRLF line ends, comments, D / F / CE / CMBLOCK
  records (a range entry included) and an underscore component that must be
  skipped: read back exactly, renumbered 1..n, and assembled through the
  model builder into the same numbering and pattern as the generated mesh.
* The reference's BENCH input (test/3d_damper/model.cdb), where the checkout
  is present: the mesh the reader builds equals the committed fixture.
* Errors: an unreadable path gives False, a malformed format line raises.
"""
import os

import numpy as np
import pytest

from nla3d_gb300 import cdb
from nla3d_gb300 import meshgen as mg
from oracle.oracle import REF_TEST

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _write_cdb(path, xyz, numbers, conn, solid=True, fixes=(), loads=(), ces=(), comps=None):
    rows = ["/COM, written by the reader test", "! a comment line",
            f"NBLOCK,6,SOLID,{len(numbers):10d},{len(numbers):10d}", "(3i9,6e21.13e3)"]
    for n, p in zip(numbers, xyz):
        # trailing zero coordinates may be omitted (the reader fills zeros)
        vals = list(p)
        while vals and vals[-1] == 0.0:
            vals.pop()
        rows.append(f"{n:9d}{0:9d}{0:9d}" + "".join(f"{v:21.13E}" for v in vals))
    rows.append("N,R5.3,LOC,       -1,")
    if solid:
        rows += [f"EBLOCK,19,SOLID,{len(conn):10d},{len(conn):10d}", "(19i9)"]
        for k, c in enumerate(conn):
            head = [1, 1, 1, 1, 0, 0, 0, 0, len(c), 0, k + 1]
            rows.append("".join(f"{v:9d}" for v in head + [numbers[i - 1] for i in c]))
    else:
        rows += [f"EBLOCK,15,,{len(conn):10d},{len(conn):10d}", "(15i9)"]
        for k, c in enumerate(conn):
            head = [k + 1, 1, 1, 1, 0]
            rows.append("".join(f"{v:9d}" for v in head + [numbers[i - 1] for i in c]))
    rows.append("       -1")
    for n, d, v in fixes:
        rows.append(f"D,{numbers[n - 1]},{cdb.DOF_LABELS[d]:<4s},{v: .8E}")
    for n, d, v in loads:
        lab = {0: "FX", 1: "FY", 2: "FZ"}[d]
        rows.append(f"F,{numbers[n - 1]},{lab},{v: .8E}")
    for k, (terms, b) in enumerate(ces):
        rows.append(f"CE,R5.0,DEFI,{len(terms):8d},{k + 1:8d},{b: .8E}")
        for s in range(0, len(terms), 2):
            part = terms[s:s + 2]
            rows.append("CE,R5.0,NODE," + ",".join(
                f"{numbers[n - 1]:10d},{cdb.DOF_LABELS[d]:<4s},{c: .8E}" for n, d, c in part))
    for name, (ctype, entries) in (comps or {}).items():
        rows += [f"CMBLOCK,{name},{ctype},{len(entries):8d}  ! component", "(8i10)"]
        for s in range(0, len(entries), 8):
            rows.append("".join(f"{v:10d}" for v in entries[s:s + 8]))
    with open(path, "wb") as fh:
        fh.write(("\r\n".join(rows) + "\r\n").encode())


@pytest.mark.parametrize("solid", [True, False])
def test_reader_round_trip(tmp_path, solid):
    mesh = mg.solid81_block(3, 2, 2, 0.5, mg.MAT_NEO_HOOKEAN, (1.0, 1000.0))
    n = mesh.n_nodes
    numbers = [10 * k + 7 for k in range(n)]             # sparse: compressNumbers renumbers
    fixes = [(1, mg.UX, 0.0), (2, mg.UZ, 0.25), (n, mg.UY, -1.5)]
    loads = [(3, mg.UX, 2.0), (4, mg.UZ, -0.5)]
    ces = [([(5, mg.UX, 1.0), (6, mg.UX, -1.0), (7, mg.UY, 0.5)], 0.1)]
    top = [k + 1 for k in range(n) if mesh.xyz[k, 2] == mesh.xyz[:, 2].max()]
    comps = {"TOP": ("NODE", [numbers[top[0] - 1], -numbers[top[2] - 1]] +
                     [numbers[t - 1] for t in top[3:]]),
             "_HIDDEN": ("NODE", [numbers[0]])}
    path = str(tmp_path / "model.cdb")
    _write_cdb(path, mesh.xyz, numbers, mesh.conn, solid, fixes, loads, ces, comps)

    md = cdb.MeshData()
    assert cdb.readCdbFile(path, md)
    assert md.nodesNumbers == numbers
    md.compressNumbers()
    assert md.nodesNumbers == list(range(1, n + 1))
    np.testing.assert_array_equal(md.nodes_array(), mesh.xyz)   # 13 digits round trip exactly here
    assert md.cellNodes == mesh.conn.tolist()
    assert md.cellIntData["TYPE"] == [1] * mesh.n_elems
    assert md.getCellsByAttribute("TYPE", 1) == list(range(mesh.n_elems))
    assert md.getDegeneratedCells() == []
    assert [(f.node, f.node_dof, f.value) for f in md.fixBcs] == fixes
    assert [(f.node, f.node_dof, f.value) for f in md.loadBcs] == loads
    assert [([(t.node, t.node_dof, t.coef) for t in m.eq], m.b) for m in md.mpcs] == ces
    # the range entry expands over the old numbers, which are 10 apart: only
    # the old numbers that name nodes map to new ones (the others map to 0,
    # as std::map::operator[] gives in the reference)
    assert set(md.feComps) == {"TOP"}
    assert md.feComps["TOP"].type == "NODE"
    lst = md.feComps["TOP"].list
    assert [v for v in lst if v] == top
    built, bfixes, bloads = cdb.to_mesh(md, mg.ELEM_SOLID81, mesh.mat_id, mesh.mat_c)
    np.testing.assert_array_equal(built.conn, mesh.conn)
    assert bfixes == fixes and bloads == loads and len(built.mpcs) == 1
    from oracle import oracle as O
    a, b = O.OracleModel(built, "port"), O.OracleModel(_with(mesh, built), "port")
    for blk in (1, 12, 2):
        for x, y in zip(a.pattern(blk), b.pattern(blk)):
            assert np.array_equal(x, y)


def _with(mesh, built):
    """The generated mesh with the constraints the reader produced."""
    mesh.fix_nodes, mesh.fix_dofs, mesh.mpcs = built.fix_nodes, built.fix_dofs, built.mpcs
    return mesh


def test_reader_errors(tmp_path):
    assert not cdb.readCdbFile(str(tmp_path / "missing.cdb"), cdb.MeshData())
    p = tmp_path / "bad.cdb"
    p.write_text("NBLOCK,6,SOLID,1,1\n(3x9)\n        1        0        0 1.0\n")
    with pytest.raises(cdb.CdbError):
        cdb.readCdbFile(str(p), cdb.MeshData())
    p.write_text("EBLOCK,19,SOLID,1,1\n(19i9)\n        1        1     12\n       -1\n")
    with pytest.raises(cdb.CdbError):
        cdb.readCdbFile(str(p), cdb.MeshData())


@pytest.mark.skipif(not os.path.isdir(REF_TEST), reason="reference tests not present")
def test_damper_cdb_builds_the_fixture_model():
    md = cdb.read_cdb(os.path.join(REF_TEST, "3d_damper", "model.cdb"))
    mesh, fixes, _ = cdb.to_mesh(md, mg.ELEM_SOLID81, mg.MAT_NEO_HOOKEAN, (10.0, 5000.0))
    g = np.load(os.path.join(GOLDEN, "damper_3d.npz"))
    np.testing.assert_array_equal(mesh.xyz, g["xyz"])
    np.testing.assert_array_equal(mesh.conn, g["conn"])
    assert np.array_equal(mesh.fix_nodes, g["fix_node"]) and np.array_equal(mesh.fix_dofs, g["fix_dof"])
    assert [f[2] for f in fixes] == g["fix_value"].tolist()
    assert len(mesh.mpcs) == len(g["mpc_b"]) == 497
    ptr = g["mpc_ptr"]
    for k, q in enumerate(mesh.mpcs):
        sl = slice(int(ptr[k]), int(ptr[k + 1]))
        assert np.array_equal(q.nodes, g["mpc_node"][sl]) and np.array_equal(q.dofs, g["mpc_dof"][sl])
        assert np.array_equal(q.coefs, g["mpc_coef"][sl]) and q.b == g["mpc_b"][k]
    assert md.feComps["TOP_SIDE"].list == g["top_side"].tolist()
