"""Generate the golden fixtures in tests/golden/ from the COMPILED REFERENCE.

Run in a checkout that has the reference sources (the oracle Makefile compiles
them into oracle/_ref/):

    python tests/golden/make_golden.py

For every case in cases.FULL_CASES it stores the equation numbers, the CSR
pattern of the three K blocks (block(1), block(1,2), block(2)), their values
and F, as produced by the reference's FEStorage::updateResults() +
assembleGlobalEqMatrices(), and seeded vectors through the reference's sparse
block products matBVprod / matBTVprod (SparseMatrix.cpp:497-558) on that K.  For cases.DIGEST_CASES (too large to commit) it
stores SHA-256 digests of the exact bytes plus a few norms.
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from oracle import oracle as O  # noqa: E402
from nla3d_gb300 import meshgen as mg  # noqa: E402
import cases  # noqa: E402


def run_reference(case):
    mesh, u, p, extra, do_update = case()
    m = O.OracleModel(mesh, "ref")
    ne, ee = m.eq_numbers()
    U = mg.u_to_vector(ne, ee, u, p, m.n_total, extra)
    m.set_U(U)
    if do_update:
        m.update()
    m.assemble()
    out = {"U": U, "node_eq": ne, "elem_eq": ee, "F": m.F(),
           "info": np.array([m.n_dofs, m.n_con, m.n_unk, m.n_mpc], np.uint32)}
    for b in (1, 12, 2):
        io, co = m.pattern(b)
        out[f"iofeir_{b}"] = io
        out[f"columns_{b}"] = co
        out[f"K_{b}"] = m.K(b)
        out[f"shape_{b}"] = np.array(m.blocks[b], np.uint32)
        if mesh.transient:
            out[f"C_{b}"] = m.C(b)
            out[f"M_{b}"] = m.M(b)
    out.update(block_products(m))
    return out


MV_PRODUCTS = ((1, 0), (2, 0), (12, 0), (12, 1))   # (block, transposed)


def block_products(m, seed=5, coef=-1.5):
    """y0 + coef * op(block) x through the model's sparse products
    (matBVprod / matBTVprod).  x is seeded N(0,1) with every 7th entry 0 and
    every 11th entry 1e-21 (below the symmetric product's 1e-20 skip)."""
    rng = np.random.default_rng(seed)
    out = {}
    for blk, trans in MV_PRODUCTS:
        rows, cols, _ = m.blocks[blk]
        nx = cols if (blk == 12 and not trans) else rows
        ny = cols if (blk == 12 and trans) else rows
        x = rng.standard_normal(nx)
        x[::7] = 0.0
        x[3::11] = 1e-21
        y0 = rng.standard_normal(ny)
        out[f"mv_{blk}_{trans}_x"] = x
        out[f"mv_{blk}_{trans}_y0"] = y0
        out[f"mv_{blk}_{trans}_y"] = m.block_mv(blk, trans, x, coef, y0)
    out["mv_coef"] = np.array(coef)
    return out


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def read_rigid_body_case(cdb_path, curve_path):
    """The reference's `rigid_body_mpc_block_ROTX` test input (test/CMakeLists.txt:51-57):
    nodes (NBLOCK), the SOLID81 connectivity (EBLOCK, last 8 fields), node
    components (CMBLOCK) and fixed DoFs (D lines) of its .cdb, plus the
    reference reaction curve (third column, test/rigid_body_mpc/)."""
    lines = open(cdb_path).read().splitlines()
    nodes, elems, comps, fixes = {}, [], {}, []
    i = 0
    while i < len(lines):
        ln = lines[i]
        if ln.startswith("NBLOCK"):
            i += 2
            while not lines[i].startswith("N,"):
                t = lines[i]
                nid = int(t[0:9])
                nodes[nid] = [float(t[27 + 20 * k: 47 + 20 * k]) for k in range(3)]
                i += 1
        elif ln.startswith("EBLOCK"):
            i += 2
            while lines[i].strip() != "-1":
                f = [int(lines[i][9 * k: 9 * k + 9]) for k in range(len(lines[i]) // 9)]
                elems.append(f[11:19])
                i += 1
        elif ln.startswith("CMBLOCK"):
            name = ln.split(",")[1].strip()
            i += 2
            comps[name] = [int(v) for v in lines[i].split()]
        elif ln.startswith("D,"):
            f = [v.strip() for v in ln.split(",")]
            fixes.append((int(f[1]), f[2], float(f[3])))
        i += 1
    curve = []
    with open(curve_path) as fh:
        next(fh)
        for row in fh:
            if row.strip():
                curve.append(float(row.split()[2]))
    return nodes, elems, comps, fixes, curve


def read_cdb(path):
    """An ANSYS .cdb through the library's reader (nla3d_gb300.cdb, which
    follows readCdbFile, FEReaders.cpp:321-729, and compressNumbers,
    FEReaders.cpp:35-80), as plain lists: node positions, cells with their
    TYPE attribute, fixed DoFs, loads, CE equations and node components."""
    from nla3d_gb300 import cdb
    md = cdb.read_cdb(path)
    return {"xyz": md.nodes_array(), "cells": md.cellNodes, "type": md.cellIntData["TYPE"],
            "fixes": [(f.node, f.node_dof, f.value) for f in md.fixBcs],
            "loads": [(f.node, f.node_dof, f.value) for f in md.loadBcs],
            "mpcs": [([(t.node, t.node_dof, t.coef) for t in m.eq], m.b) for m in md.mpcs],
            "comps": {k: list(v.list) for k, v in md.feComps.items()}}


def read_ref_curve(path):
    """main.cpp readRefCurveData: the third column, consecutive repeats dropped."""
    out, prev = [], -1.0
    with open(path) as fh:
        next(fh)
        for row in fh:
            if row.strip():
                v = float(row.split()[2])
                if v != prev:
                    out.append(v)
                    prev = v
    return out


def write_damper_fixture():
    """The reference's 3d_damper BENCH input (test/CMakeLists.txt:148-153):
    SOLID81 on the TYPE 1 elements of model.cdb, its fixed DoFs (with their
    end values), its 497 CE equations, the TOP_SIDE node component used for
    the UY reaction, and the ANSYS loading curve (test/3d_damper/ansys/)."""
    base = os.path.join(O.REF_TEST, "3d_damper")
    md = read_cdb(f"{base}/model.cdb")
    conn = np.array([c for c, t in zip(md["cells"], md["type"]) if t == 1], dtype=np.uint32)
    terms = [t for terms, _ in md["mpcs"] for t in terms]
    np.savez_compressed(
        os.path.join(HERE, "damper_3d.npz"),
        xyz=md["xyz"], conn=conn,
        fix_node=np.array([f[0] for f in md["fixes"]], dtype=np.uint32),
        fix_dof=np.array([f[1] for f in md["fixes"]], dtype=np.int32),
        fix_value=np.array([f[2] for f in md["fixes"]], dtype=np.float64),
        mpc_ptr=np.cumsum([0] + [len(t) for t, _ in md["mpcs"]]).astype(np.uint32),
        mpc_node=np.array([t[0] for t in terms], dtype=np.uint32),
        mpc_dof=np.array([t[1] for t in terms], dtype=np.int32),
        mpc_coef=np.array([t[2] for t in terms], dtype=np.float64),
        mpc_b=np.array([b for _, b in md["mpcs"]], dtype=np.float64),
        top_side=np.array(md["comps"]["TOP_SIDE"], dtype=np.uint32),
        ref_curve=np.array(read_ref_curve(f"{base}/ansys/loading_curve_ansys.txt")))
    print("wrote damper_3d", conn.shape, len(md["mpcs"]), "CE,", len(md["fixes"]), "D")


def write_a2000_fixture():
    """The reference's a2000_damper BENCH input (test/CMakeLists.txt:141-146):
    PLANE41 on the TYPE 1 elements of a2000.cdb, its fixed DoFs, the DISP_BC
    node component of the UY reaction, and the ANSYS loading curve."""
    base = os.path.join(O.REF_TEST, "a2000_damper")
    md = read_cdb(f"{base}/a2000.cdb")
    conn = np.array([c for c, t in zip(md["cells"], md["type"]) if t == 1], dtype=np.uint32)
    assert not md["mpcs"]
    np.savez_compressed(
        os.path.join(HERE, "a2000_plane41.npz"),
        xyz=md["xyz"], conn=conn,
        fix_node=np.array([f[0] for f in md["fixes"]], dtype=np.uint32),
        fix_dof=np.array([f[1] for f in md["fixes"]], dtype=np.int32),
        fix_value=np.array([f[2] for f in md["fixes"]], dtype=np.float64),
        disp_bc=np.array(md["comps"]["DISP_BC"], dtype=np.uint32),
        ref_curve=np.array(read_ref_curve(f"{base}/ansys/loading_curve_ansys.txt")))
    print("wrote a2000_plane41", conn.shape, len(md["fixes"]), "D")


def write_heat_fixture():
    """The reference's QUADTH_test / QUADTH_transient inputs (test/QUADTH):
    the QUADTH (TYPE 1) and SurfaceLINETH (TYPE 2) cells of heat.cdb, its
    HEAT loads, the PROBE node, and the ANSYS results the two tests check:
    every node's steady temperature (temp.txt) and the probe's transient
    history (temphistory.txt)."""
    base = os.path.join(O.REF_TEST, "QUADTH")
    md = read_cdb(f"{base}/heat.cdb")
    quads = np.array([c for c, t in zip(md["cells"], md["type"]) if t == 1], dtype=np.uint32)
    lines = np.array([c for c, t in zip(md["cells"], md["type"]) if t == 2], dtype=np.uint32)
    temp = []
    with open(f"{base}/temp.txt", encoding="latin-1") as fh:
        next(fh)
        for row in fh:
            if row.strip():
                temp.append(float(row.split()[1]))
    hist_t, hist_v = [], []
    with open(f"{base}/temphistory.txt") as fh:
        next(fh)
        for row in fh:
            if row.strip():
                a, b = row.split(",")
                hist_t.append(float(a))
                hist_v.append(float(b))
    assert len(temp) == md["xyz"].shape[0] and not md["fixes"]
    np.savez_compressed(
        os.path.join(HERE, "heat_quadth.npz"),
        xyz=md["xyz"], quads=quads, lines=lines,
        load_node=np.array([f[0] for f in md["loads"]], dtype=np.uint32),
        load_dof=np.array([f[1] for f in md["loads"]], dtype=np.int32),
        load_value=np.array([f[2] for f in md["loads"]], dtype=np.float64),
        probe=np.array(md["comps"]["PROBE"], dtype=np.uint32),
        ansys_temp=np.array(temp), ansys_time=np.array(hist_t), ansys_probe=np.array(hist_v))
    print("wrote heat_quadth", quads.shape, lines.shape, len(md["loads"]), "F")


VTK_CASES = ("bar_mpc_2x2x3", "quadth_lines_6x5", "plane41_nh_3x2", "tetra0_3x3x3")


def vtk_state(name):
    """The state the VTK fixtures are written from: the case's vecU and a
    deterministic vecR."""
    mesh, u, p, extra, do_update = cases.FULL_CASES[name]()
    m = O.OracleModel(mesh, "port")
    ne, ee = m.eq_numbers()
    U = mg.u_to_vector(ne, ee, u, p, m.n_total, extra)
    R = np.linspace(-1.5, 2.5, m.n_total) ** 3
    return mesh, U, R


def write_vtk_fixtures():
    """The reference's own VtkProcessor output (pre() + process(7)) for a few
    cases, as text fixtures vtk_<case>_<0|7>.vtk."""
    import tempfile
    for name in VTK_CASES:
        mesh, U, R = vtk_state(name)
        m = O.OracleModel(mesh, "ref")
        with tempfile.TemporaryDirectory() as d:
            prefix = os.path.join(d, "out")
            m.write_vtk(prefix, 7, U, R)
            for step in (0, 7):
                with open(f"{prefix}{step}.vtk") as fh, \
                        open(os.path.join(HERE, f"vtk_{name}_{step}.vtk"), "w") as out:
                    out.write(fh.read())
        print("wrote vtk", name)


def write_tetra0_fixture():
    """The reference's TETRA0_test input (test/TETRA0): the TYPE 1 cells of
    tetra.cdb as TETRA0 (nodes 0, 1, 2, 4 of the degenerate 8-node cell, as
    TETRA0_test.cpp takes them), its D fixes and F loads, and the ANSYS
    results the test checks: nodal displacements (disp.res, 1e-10) and
    element stresses (stress.res, 1e-3)."""
    base = os.path.join(O.REF_TEST, "TETRA0")
    md = read_cdb(f"{base}/tetra.cdb")
    conn = np.array([[c[0], c[1], c[2], c[4]] for c, t in zip(md["cells"], md["type"]) if t == 1],
                    dtype=np.uint32)

    def table(path, cols):
        rows = []
        with open(path) as fh:
            next(fh)
            for row in fh:
                if row.strip():
                    rows.append([float(v) for v in row.split()[1:1 + cols]])
        return np.array(rows)
    np.savez_compressed(
        os.path.join(HERE, "tetra0_ansys.npz"),
        xyz=md["xyz"], conn=conn,
        fix_node=np.array([f[0] for f in md["fixes"]], dtype=np.uint32),
        fix_dof=np.array([f[1] for f in md["fixes"]], dtype=np.int32),
        fix_value=np.array([f[2] for f in md["fixes"]], dtype=np.float64),
        load_node=np.array([f[0] for f in md["loads"]], dtype=np.uint32),
        load_dof=np.array([f[1] for f in md["loads"]], dtype=np.int32),
        load_value=np.array([f[2] for f in md["loads"]], dtype=np.float64),
        ansys_disp=table(f"{base}/disp.res", 3), ansys_stress=table(f"{base}/stress.res", 6))
    print("wrote tetra0_ansys", conn.shape, len(md["fixes"]), "D", len(md["loads"]), "F")


def write_rigid_body_fixture():
    base = os.path.join(O.REF_TEST, "rigid_body_mpc")
    nodes, elems, comps, fixes, curve = read_rigid_body_case(
        f"{base}/block_ROTX.cdb", f"{base}/reference_MOMZ_reaction.txt")
    labels = ["UX", "UY", "UZ", "ROTX", "ROTY", "ROTZ", "HYDRO_PRESSURE", "TEMP"]
    n = max(nodes)
    xyz = np.array([nodes[k] for k in range(1, n + 1)], dtype=np.float64)
    np.savez_compressed(
        os.path.join(HERE, "rigid_body_mpc_block_rotx.npz"),
        xyz=xyz, conn=np.array(elems, dtype=np.uint32),
        top_side=np.array(comps["TOP_SIDE"], dtype=np.uint32),
        master=np.array(comps["MASTER_NODE"], dtype=np.uint32),
        fix_node=np.array([f[0] for f in fixes], dtype=np.uint32),
        fix_dof=np.array([labels.index(f[1]) for f in fixes], dtype=np.int32),
        fix_value=np.array([f[2] for f in fixes], dtype=np.float64),
        ref_curve=np.array(curve, dtype=np.float64))
    print("wrote rigid_body_mpc_block_rotx")


def main():
    write_rigid_body_fixture()
    write_damper_fixture()
    write_a2000_fixture()
    write_heat_fixture()
    write_tetra0_fixture()
    if not O.build_ref():
        sys.exit("reference sources not found; cannot regenerate goldens")
    write_vtk_fixtures()
    for name, case in cases.FULL_CASES.items():
        out = run_reference(case)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        print("wrote", name)
    lines = []
    for name, case in cases.DIGEST_CASES.items():
        out = run_reference(case)
        for k in sorted(out):
            lines.append(f"{name} {k} {digest(out[k])}")
        lines.append(f"{name} normK2 {float(np.abs(out['K_2']).max()):.17g}")
        lines.append(f"{name} normF {float(np.abs(out['F']).max()):.17g}")
        print("digested", name)
    with open(os.path.join(HERE, "digests.txt"), "w") as f:
        f.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
