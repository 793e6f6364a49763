"""Pin the CPU oracle (oracle/nla3d_oracle.c) before it is trusted.

* bit-exact against the committed golden fixtures, which were produced by the
  reference's own compiled sources (tests/golden/make_golden.py);
* bit-exact against the compiled reference live, on extra seeded cases, when
  the reference checkout is present;
* the reference's own known-answer tests: the mat_prod MATLAB vectors
  (test/mat_prod_test.cpp, eps 1e-6) and the isoparametric hexahedron
  invariants (test/isoparametric_test.cpp:280-447).
"""
import hashlib
import os

import numpy as np
import pytest

import cases
from nla3d_gb300 import meshgen as mg
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
from oracle.oracle import REF_TEST  # noqa: E402


def _run(kind, case):
    mesh, u, p, extra, do_update = case()
    m = O.OracleModel(mesh, kind)
    ne, ee = m.eq_numbers()
    U = mg.u_to_vector(ne, ee, u, p, m.n_total, extra)
    m.set_U(U)
    if do_update:
        m.update()
    m.assemble()
    return m, U, ne, ee


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint64)


@pytest.mark.parametrize("name", sorted(cases.FULL_CASES))
def test_port_matches_reference_goldens_bit_exact(name):
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    m, U, ne, ee = _run("port", cases.FULL_CASES[name])
    assert np.array_equal(ne, g["node_eq"]) and np.array_equal(ee, g["elem_eq"])
    assert np.array_equal(_bits(U), _bits(g["U"]))
    for b in (1, 12, 2):
        io, co = m.pattern(b)
        assert tuple(m.blocks[b]) == tuple(g[f"shape_{b}"])
        assert np.array_equal(io, g[f"iofeir_{b}"])
        assert np.array_equal(co, g[f"columns_{b}"])
        assert np.array_equal(_bits(m.K(b)), _bits(g[f"K_{b}"])), f"K block {b}"
        if f"C_{b}" in g:
            assert np.array_equal(_bits(m.C(b)), _bits(g[f"C_{b}"])), f"C block {b}"
            assert np.array_equal(_bits(m.M(b)), _bits(g[f"M_{b}"])), f"M block {b}"
    assert np.array_equal(_bits(m.F()), _bits(g["F"]))


MV_PRODUCTS = ((1, 0), (2, 0), (12, 0), (12, 1))


@pytest.mark.parametrize("name", sorted(cases.FULL_CASES))
def test_port_block_products_match_reference_goldens(name):
    """matBVprod / matBTVprod (SparseMatrix.cpp:497-558) on the assembled K:
    the port gives the compiled reference's vectors bit for bit."""
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    m = _run("port", cases.FULL_CASES[name])[0]
    coef = float(g["mv_coef"])
    for blk, trans in MV_PRODUCTS:
        y = m.block_mv(blk, trans, g[f"mv_{blk}_{trans}_x"], coef, g[f"mv_{blk}_{trans}_y0"])
        assert np.array_equal(_bits(y), _bits(g[f"mv_{blk}_{trans}_y"])), (blk, trans)


def test_port_matches_reference_digests_cube10():
    want = {}
    with open(os.path.join(GOLDEN, "digests.txt")) as f:
        for line in f:
            case, key, val = line.split()
            want[(case, key)] = val
    m, U, ne, ee = _run("port", cases.cube10_nh)
    got = {"U": U, "node_eq": ne, "elem_eq": ee, "F": m.F()}
    for b in (1, 12, 2):
        io, co = m.pattern(b)
        got[f"iofeir_{b}"], got[f"columns_{b}"], got[f"K_{b}"] = io, co, m.K(b)
        got[f"shape_{b}"] = np.array(m.blocks[b], np.uint32)
    got["info"] = np.array([m.n_dofs, m.n_con, m.n_unk, m.n_mpc], np.uint32)
    rng = np.random.default_rng(5)
    for blk, trans in MV_PRODUCTS:
        rows, cols, _ = m.blocks[blk]
        nx = cols if (blk == 12 and not trans) else rows
        ny = cols if (blk == 12 and trans) else rows
        x = rng.standard_normal(nx)
        x[::7] = 0.0
        x[3::11] = 1e-21
        y0 = rng.standard_normal(ny)
        got[f"mv_{blk}_{trans}_x"], got[f"mv_{blk}_{trans}_y0"] = x, y0
        got[f"mv_{blk}_{trans}_y"] = m.block_mv(blk, trans, x, -1.5, y0)
    got["mv_coef"] = np.array(-1.5)
    assert m.blocks[2] == (4993, 4993, 161056)
    for k, v in got.items():
        assert hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest() == \
            want[("cube10_nh", k)], k


@pytest.mark.skipif(not O.ref_available(), reason="compiled reference not present")
@pytest.mark.parametrize("seed", [11, 12, 13])
def test_port_matches_compiled_reference_live(seed):
    rng = np.random.default_rng(seed)
    nx, ny, nz = (int(v) for v in rng.integers(1, 5, size=3))
    mat = [(mg.MAT_NEO_HOOKEAN, (1.3, 700.0)), (mg.MAT_MOONEY_RIVLIN, (0.3, 0.2, 1500.0)),
           (mg.MAT_BIDERMAN, (0.4, 0.03, 0.002, 0.05, 900.0))][seed % 3]
    mesh = mg.solid81_block(nx, ny, nz, 0.3, mat[0], mat[1], clamp_z0=bool(seed % 2))
    u, p = mg.twist_state(mesh, angle_deg=20.0, stretch=1.4, noise_frac=0.02, seed=seed)
    case = lambda: (mesh, u, p, None, True)  # noqa: E731
    a = _run("port", case)[0]
    b = _run("ref", case)[0]
    for blk in (1, 12, 2):
        assert np.array_equal(_bits(a.K(blk)), _bits(b.K(blk)))
    assert np.array_equal(_bits(a.F()), _bits(b.F()))


def test_max_in_row_overflow_is_reported():
    # 1681-slave style overflow (SparseMatrix.cpp:84): a small row capacity trips it.
    mesh = mg.solid81_bar_mpc(2, 2, 2, 1.0)
    with pytest.raises(O.OracleError, match="maxInRow overflow"):
        O.OracleModel(mesh, "port", max_in_row=8)


def _read_mat_prod(fname):
    with open(os.path.join(REF_TEST, "mat_prod", "matlab", fname)) as f:
        return np.array(f.read().split(), dtype=np.float64)


@pytest.mark.skipif(not os.path.isdir(REF_TEST), reason="reference tests not present")
def test_mat_prod_known_answers():
    """test/mat_prod_test.cpp: 100 cases per product, eps 1e-6."""
    import ctypes
    lib = O.port_lib()
    p = lambda a: a.ctypes.data  # noqa: E731
    eps = 1e-6
    # matBVprod 24x9
    v = _read_mat_prod("matBVprod_2409").reshape(100, -1)
    for row in v:
        B, V, Rf = row[:216], row[216:225], row[225:249]
        R = np.zeros(24)
        lib.orc_matBVprod(24, 9, p(B), p(V), 1.0, p(R))
        assert np.abs(R - Rf).max() <= eps
    v = _read_mat_prod("matBTVprod_2409").reshape(100, -1)
    for row in v:
        B, V, Rf = row[:216], row[216:240], row[240:249]
        R = np.zeros(9)
        lib.orc_matBTVprod(24, 9, p(B), p(V), 1.0, p(R))
        assert np.abs(R - Rf).max() <= eps
    v = _read_mat_prod("matABprod_240912").reshape(100, -1)
    for row in v:
        A, B, Rf = row[:216], row[216:324], row[324:612]
        R = np.zeros(288)
        lib.orc_matABprod(24, 9, 12, p(A), p(B), 1.0, p(R))
        assert np.abs(R - Rf).max() <= eps
    v = _read_mat_prod("matATBprod_240912").reshape(100, -1)
    for row in v:
        A, B, Rf = row[:216], row[216:504], row[504:612]
        R = np.zeros(108)
        lib.orc_matATBprod(24, 9, 12, p(A), p(B), 1.0, p(R))
        assert np.abs(R - Rf).max() <= eps
    v = _read_mat_prod("matBTDBprod_2409").reshape(100, -1)
    for row in v:
        B, D, Rf = row[:216], row[216:216 + 300], row[516:561]
        R = np.zeros(45)
        lib.orc_matBTDBprod(24, 9, p(B), p(D), 1.0, p(R))
        assert np.abs(R - Rf).max() <= eps
    del ctypes


def _hex(nodes):
    lib = O.port_lib()
    X = np.ascontiguousarray(nodes, dtype=np.float64)
    G = np.zeros((27, 8, 3))
    det = np.zeros(27)
    out = []
    for order in (1, 2, 3):
        lib.orc_hex_jacobian(X.ctypes.data, order, G.ctypes.data, det.ctypes.data)
        npnt = {1: 1, 2: 8, 3: 27}[order]
        w = {1: [8.0], 2: [1.0] * 8}.get(order)
        out.append((G[:npnt].copy(), det[:npnt].copy(), npnt))
    return out


def test_isoparametric_hexahedron_invariants():
    """test/isoparametric_test.cpp:280-447: det J = 1 on the reference cube,
    2 when stretched x2, volume 8 / 16, invariance under translation."""
    cube = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                     [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], float)
    stretched = cube * np.array([2.0, 1.0, 1.0])
    arb = np.array([[-12, 1, -7], [4, -5, -7], [7, 1, -7], [-2, 3, -7],
                    [-12, 1, 4], [4, -5, 4], [7, 1, 4], [-2, 3, 4]], float)
    moved = arb + np.array([9.0, -5.0, 2.0])
    th = 1e-10
    for (G, det, n) in _hex(cube):
        assert np.allclose(det, 1.0, atol=th)
    weights = {1: np.array([8.0]), 8: np.ones(8)}
    for (G, det, n) in _hex(stretched):
        assert np.allclose(det, 2.0, atol=th)
        if n in weights:
            assert abs(float((weights[n] * det).sum()) - 16.0) < th
    for (Ga, da, n), (Gb, db, _) in zip(_hex(arb), _hex(moved)):
        assert np.allclose(da, db, atol=th) and np.allclose(Ga, Gb, atol=th)


def test_thermal_goldens_exercise_every_term():
    """The QUADTH fixtures are not vacuous: volume flux, convection lines
    (F and K on the line nodes) and the capacity matrix all contribute, and
    the second environment temperature of a line with etemp[1] = 0 is taken
    from etemp[0] (SurfaceLINETH::pre)."""
    mesh = cases.quadth_lines_6x5()[0]
    assert mesh.lines.n == 11 and (mesh.elem_params[:, 1] != 0).any()
    g = np.load(os.path.join(GOLDEN, "quadth_lines_6x5.npz"))
    base = mesh.__class__(**{**mesh.__dict__, "lines": None})
    m0 = O.OracleModel(base, "port")
    m0.set_U(np.zeros(m0.n_total))
    m0.assemble()
    assert not np.array_equal(m0.F(), g["F"])            # lines load F
    assert not np.array_equal(m0.K(2), g["K_2"])         # convection adds to K
    t = cases.quadth_transient_5x4()[0]
    gt = np.load(os.path.join(GOLDEN, "quadth_transient_5x4.npz"))
    assert np.abs(gt["C_2"]).max() > 0 and not np.any(gt["M_2"])
    # a zero second temperature equals giving it explicitly
    lines = t.lines
    et = lines.etemp.copy()
    et[et[:, 1] == 0.0, 1] = et[et[:, 1] == 0.0, 0]
    t2 = t.__class__(**{**t.__dict__, "lines": lines.__class__(lines.conn, lines.htc, lines.flux,
                                                                et)})
    m2 = O.OracleModel(t2, "port")
    m2.set_U(np.zeros(m2.n_total))
    m2.assemble()
    assert np.array_equal(_bits(m2.F()), _bits(gt["F"]))
