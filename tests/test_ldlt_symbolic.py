"""Symbolic analysis of the device LDL^T (nla3d_ldlt_analyze, host only):
the supernodal structure holds every fill entry.  A dense emulation of the
multifrontal algorithm the device runs (scatter, extend-add into the parent
front, partial LDL^T of the pivots) on the structure the library returns
reproduces P K P^T = L D L^T for the K(2) blocks of the oracle's assembled
cases (u/p, MPC equations ordered last, thermal)."""
import numpy as np
import pytest

import cases
from nla3d_gb300 import ldlt
from nla3d_gb300 import meshgen as mg
from nla3d_gb300.newton import csr_full, nested_dissection
from oracle import oracle as O


def _k2(name):
    mesh, u, p, extra, do_update = cases.FULL_CASES[name]()
    m, U, K, F = O.solve_state(mesh, u, p, "port", extra)
    io, co = m.pattern(2)
    rows, cols, _ = m.blocks[2]
    A = csr_full(io, co, K[2], rows, cols, True).toarray()
    return m, io, co, A


def _emulate(A, sym):
    """Multifrontal LDL^T on the returned structure; returns (L, D) in factor order."""
    n = A.shape[0]
    perm = sym["perm"]
    PA = A[np.ix_(perm, perm)]
    sn_first, row_ptr, rows = sym["sn_first"], sym["row_ptr"], sym["rows"]
    ns = sn_first.size - 1
    col2sn = np.repeat(np.arange(ns), np.diff(sn_first))
    parent = np.full(ns, -1)
    for s in range(ns):
        last = sn_first[s + 1] - 1
        r = rows[row_ptr[s]:row_ptr[s + 1]]
        k = sn_first[s + 1] - sn_first[s]
        if r.size > k:
            parent[s] = col2sn[r[k]]
    fronts, upd = {}, {}
    L = np.zeros((n, n))
    D = np.zeros(n)
    for s in range(ns):
        r = rows[row_ptr[s]:row_ptr[s + 1]]
        f, k, m = sn_first[s], sn_first[s + 1] - sn_first[s], r.size
        assert np.array_equal(r[:k], np.arange(f, f + k)) and np.all(np.diff(r) > 0)
        pos = {int(x): i for i, x in enumerate(r)}
        F = np.zeros((m, m))
        # original entries of the pivot columns (lower part)
        for c in range(k):
            col = f + c
            nz = np.nonzero(PA[col:, col])[0] + col
            for i in nz:
                assert int(i) in pos, "matrix entry outside its front"
                F[pos[int(i)], c] = PA[i, col]
        for c_sn in [c for c in range(s) if parent[c] == s]:
            rc, U = upd.pop(c_sn)
            idx = [pos[int(x)] for x in rc]     # KeyError: child row missing from the parent
            F[np.ix_(idx, idx)] += U
        for p in range(k):
            d = F[p, p]
            w = F[p + 1:, p].copy()
            F[p + 1:, p] = w / d
            F[p + 1:, p + 1:] -= np.outer(F[p + 1:, p], w)
            D[f + p] = d
        L[np.ix_(r, np.arange(f, f + k))] = np.tril(F[:, :k], -1)[:, :k] if m else 0
        upd[s] = (r[k:], np.tril(F[k:, k:]) + np.tril(F[k:, k:], -1).T)
    L += np.eye(n)
    return PA, L, D


@pytest.mark.parametrize("name", ["cube4_nh_clamped", "mr_twist_3x2x4", "bar_mpc_2x2x3",
                                  "ce_block_3x3x2", "plane41_nh_3x2", "tetra0_3x3x3",
                                  "quadth_lines_6x5"])
@pytest.mark.parametrize("order", ["identity", "nd"])
def test_structure_holds_the_factor(name, order):
    m, io, co, A = _k2(name)
    n = A.shape[0]
    perm = None
    if order == "nd":
        pts = np.random.default_rng(0).random((n, 3))
        K = csr_full(io, co, np.ones(co.size), n, n, True)
        perm = ldlt.saddle_order(io, co, nested_dissection(K, pts, leaf=8), m.n_unk)
    else:
        perm = ldlt.saddle_order(io, co, np.arange(n), m.n_unk)
    sym = ldlt.analyze(io, co, perm)
    assert np.array_equal(np.sort(sym["perm"]), np.arange(n))
    PA, L, D = _emulate(A, sym)
    R = L @ np.diag(D) @ L.T
    assert np.abs(R - PA).max() <= 1e-9 * np.abs(PA).max()
    # every structural nonzero of the exact factor lies in the structure
    assert sym["nnz_L"] >= int(np.count_nonzero(np.abs(np.tril(L)) > 0))


def test_analyze_rejects_bad_input():
    io = np.array([1, 2, 3], np.uint32)
    co = np.array([1, 2], np.uint32)
    with pytest.raises(Exception):
        ldlt.analyze(io, co, np.array([0, 0], np.int32))     # not a permutation
    with pytest.raises(Exception):
        ldlt.analyze(np.array([1, 2, 3], np.uint32), np.array([2, 1], np.uint32))  # lower entry


def test_sizes_of_a_larger_mesh():
    """A 12^3 SOLID81 block with the geometric nested-dissection order: the
    factor is smaller and cheaper than with the natural (banded) order."""
    mesh = mg.solid81_block(12, 12, 12, 1.0 / 12, clamp_z0=True)
    o = O.OracleModel(mesh, "port")
    io, co = o.pattern(2)
    n = io.size - 1
    ne, ee = o.eq_numbers()
    xyz = mesh.xyz
    cen = xyz[mesh.conn.astype(np.int64) - 1].mean(axis=1)
    pts = np.zeros((n, 3))
    for d in range(8):
        eq = ne[:, d].astype(np.int64)
        sel = eq > o.n_con
        pts[eq[sel] - o.n_con - 1] = xyz[sel]
        eqe = ee[:, d].astype(np.int64)
        sele = eqe > o.n_con
        pts[eqe[sele] - o.n_con - 1] = cen[sele]
    K = csr_full(io, co, np.ones(co.size), n, n, True)
    nd = ldlt.analyze(io, co, nested_dissection(K, pts).astype(np.int32))
    nat = ldlt.analyze(io, co)
    assert nd["nnz_L"] < 0.8 * nat["nnz_L"] and nd["flops"] < 0.6 * nat["flops"]
    assert nd["levels"] > 3 and nd["supernodes"] < n


@pytest.mark.parametrize("name", ["bar_mpc_2x2x3", "bar_mpc_ce_2x2x3", "cube4_nh_clamped",
                                  "plane41_nh_3x2", "quadth_5x4", "block_14"])
def test_library_order_equals_the_python_nested_dissection(name):
    """nla3d_ldlt_order (the drivers' order, computed in the library) is
    exactly saddle_order(nested_dissection(...)) of the Python restatement."""
    from nla3d_gb300.newton import row_points
    from nla3d_gb300.storage import FEStorage
    mesh = (mg.solid81_block(14, 14, 14, 1.0 / 14, clamp_z0=True) if name == "block_14"
            else cases.FULL_CASES[name]()[0])
    s = FEStorage(mesh).buildPattern()
    io, co = s.pattern(2)
    n = io.size - 1
    pts = row_points(s, s.n_con, s.n_unk, s.n_mpc)
    K = csr_full(io, co, np.ones(co.size), n, n, True)
    want = ldlt.saddle_order(io, co, nested_dissection(K, pts), s.n_unk)
    assert np.array_equal(ldlt.fill_reducing_order(io, co, pts, s.n_unk), want)


def test_order_and_host_solve_reject_bad_input():
    """nla3d_ldlt_order and nla3d_ldlt_solve_host return NLA3D_ERR_ARG on
    bad arguments (no GPU needed)."""
    import ctypes
    from nla3d_gb300 import _lib
    lib = _lib.load()
    ERR_ARG = 1
    io = np.array([1, 2, 3], np.uint32)
    co = np.array([1, 2], np.uint32)
    pts = np.zeros((2, 3))
    out = np.zeros(2, np.int32)
    p = lambda a: a.ctypes.data  # noqa: E731
    assert lib.nla3d_ldlt_order(2, p(io), p(co), None, 2, p(out)) == ERR_ARG
    assert lib.nla3d_ldlt_order(0, p(io), p(co), p(pts), 2, p(out)) == ERR_ARG
    bad = np.array([2, 1], np.uint32)   # row 2 names column 1: not upper
    assert lib.nla3d_ldlt_order(2, p(io), p(bad), p(pts), 2, p(out)) == ERR_ARG
    assert lib.nla3d_ldlt_order(2, p(io), p(co), p(pts), 2, p(out)) == 0
    assert sorted(out.tolist()) == [0, 1]
    assert lib.nla3d_ldlt_solve_host(None, None, None, None, 1, 1e-10, None, None) == \
        ERR_ARG
    with pytest.raises(ValueError):
        ldlt.fill_reducing_order(io, co, np.zeros((3, 3)), 2)
