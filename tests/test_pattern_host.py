"""Host side of libnla3d_gpu.so (no GPU needed): DoF numbering, the block CSR
pattern and the element -> slot maps, checked against the reference's own
outputs (golden fixtures from the compiled reference, and the oracle)."""
import os

import numpy as np
import pytest

import cases
from nla3d_gb300 import meshgen as mg
from nla3d_gb300.storage import FEStorage
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _host(mesh):
    return FEStorage(mesh).buildPattern()


@pytest.mark.parametrize("name", sorted(cases.FULL_CASES))
def test_numbering_and_pattern_bit_exact_vs_reference(name):
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    mesh = cases.FULL_CASES[name]()[0]
    s = _host(mesh)
    ne, ee = s.eq_numbers()
    assert np.array_equal(ne, g["node_eq"]) and np.array_equal(ee, g["elem_eq"])
    assert [s.n_dofs, s.n_con, s.n_unk, s.n_mpc] == list(g["info"])
    for b in (1, 12, 2):
        assert s.blocks[b] == tuple(int(v) for v in g[f"shape_{b}"])
        io, co = s.pattern(b)
        assert np.array_equal(io, g[f"iofeir_{b}"]), b
        assert np.array_equal(co, g[f"columns_{b}"]), b


def test_pattern_cube10_matches_oracle():
    mesh = cases.cube10_nh()[0]
    s = _host(mesh)
    o = O.OracleModel(mesh, "port")
    assert s.blocks[2] == (4993, 4993, 161056)
    for b in (1, 12, 2):
        a, c = s.pattern(b), o.pattern(b)
        assert np.array_equal(a[0], c[0]) and np.array_equal(a[1], c[1])


@pytest.mark.parametrize("nx,ny,nz,clamp", [(2, 3, 4, True), (5, 1, 2, False), (3, 3, 3, True)])
def test_pattern_random_blocks_match_oracle(nx, ny, nz, clamp):
    mesh = mg.solid81_block(nx, ny, nz, 0.5, clamp_z0=clamp)
    s = _host(mesh)
    o = O.OracleModel(mesh, "port")
    for b in (1, 12, 2):
        a, c = s.pattern(b), o.pattern(b)
        assert np.array_equal(a[0], c[0]) and np.array_equal(a[1], c[1])


def _slot_rowcol(s):
    """(row, col) global equation pair of every slot of the concatenated K values."""
    rows, cols = [], []
    nc = s.n_con
    for b in (1, 12, 2):
        io, co = s.pattern(b)
        r = np.repeat(np.arange(1, io.size, dtype=np.int64), np.diff(io.astype(np.int64)))
        c = co.astype(np.int64)
        if b == 1:
            rows.append(r); cols.append(c)
        elif b == 12:
            rows.append(r); cols.append(c + nc)
        else:
            rows.append(r + nc); cols.append(c + nc)
    return np.concatenate(rows), np.concatenate(cols)


@pytest.mark.parametrize("name", ["cube4_nh_clamped", "bar_mpc_2x2x3", "tetra0_3x3x3",
                                  "quadth_5x4"])
def test_slot_maps_point_at_the_reference_entries(name):
    mesh = cases.FULL_CASES[name]()[0]
    s = _host(mesh)
    ne, ee = s.eq_numbers()
    ks, fs = s.slot_maps()
    srow, scol = _slot_rowcol(s)
    npe = mesh.conn.shape[1]
    conn = mesh.conn.astype(np.int64) - 1
    if mesh.elem_type == mg.ELEM_SOLID81:
        pairs = []
        for i in range(8):
            for di in range(3):
                for j in range(i, 8):
                    for dj in range(3):
                        if i == j and dj < di:
                            continue
                        pairs.append((i, di, j, dj))
        pairs += [(i, di, -1, 6) for i in range(8) for di in range(3)] + [(-1, 6, -1, 6)]
        fpairs = [(i, di) for i in range(8) for di in range(3)] + [(-1, 6)]
    else:
        nd = 1 if mesh.elem_type == mg.ELEM_QUADTH else 3
        pairs = []
        for i in range(npe):
            for di in range(nd):
                for j in range(i, npe):
                    for dj in range(nd):
                        if i == j and dj < di:
                            continue
                        t = (7, 7) if nd == 1 else (di, dj)
                        pairs.append((i, t[0], j, t[1]))
        fpairs = [(i, 7) for i in range(npe)] if nd == 1 else []
    assert ks.shape[1] == len(pairs) and fs.shape[1] == len(fpairs)
    E = mesh.n_elems

    def eq(ent, t):
        if ent < 0:
            return ee[np.arange(E), t].astype(np.int64)
        return ne[conn[:, ent], t].astype(np.int64)

    for c, (a, ta, b, tb) in enumerate(pairs):
        i, j = eq(a, ta), eq(b, tb)
        lo, hi = np.minimum(i, j), np.maximum(i, j)
        assert np.array_equal(srow[ks[:, c]], lo) and np.array_equal(scol[ks[:, c]], hi)
    for c, (a, ta) in enumerate(fpairs):
        assert np.array_equal(fs[:, c].astype(np.int64), eq(a, ta) - 1)


def test_bad_mesh_is_rejected_without_crash():
    mesh = mg.solid81_block(2, 2, 2)
    mesh.conn = mesh.conn.copy()
    mesh.conn[0, 0] = mesh.n_nodes + 5
    s = FEStorage(mesh)
    with pytest.raises(RuntimeError, match="missing node"):
        s.buildPattern()
