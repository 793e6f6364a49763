"""GPU parity of the assembly path through the C ABI (libnla3d_gpu.so).

Tolerance (FP64 path): max |K_gpu - K_ref| / max |K_ref| <= 1e-12 per K block
and the same for F, against (a) the committed fixtures produced by the
reference's own compiled sources and (b) the bit-exact CPU oracle.  The mixed
path computes F_u in float-pair arithmetic and the volumetric terms (J, K_up,
K_pp, F_p) in FP64, all held to the same 1e-12 bound, and K_uu in FP32
(within 2e-5).
"""
import os

import numpy as np
import pytest

import cases
from nla3d_gb300 import meshgen as mg
from nla3d_gb300.storage import FEStorage, assemble_state
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL_FP64 = 1e-12
TOL_MIXED_K = 2e-5


def rel(a, b):
    if b.size == 0:
        return 0.0
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _gpu(case, precision="fp64"):
    mesh, u, p, extra, do_update = case()
    return assemble_state(mesh, u, p, precision, extra, do_update)


@pytest.mark.parametrize("name", sorted(cases.FULL_CASES))
def test_fp64_matches_reference_fixtures(name):
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    s, U, K, F = _gpu(cases.FULL_CASES[name])
    assert np.array_equal(U, g["U"])
    for b in (1, 12, 2):
        assert rel(K[b], g[f"K_{b}"]) <= TOL_FP64, (b, rel(K[b], g[f"K_{b}"]))
    assert rel(F, g["F"]) <= TOL_FP64, rel(F, g["F"])
    for b in (1, 12, 2):
        if f"C_{b}" in g:   # transient: capacity C and mass M on K's pattern
            assert rel(s.C(b), g[f"C_{b}"]) <= TOL_FP64, (b, rel(s.C(b), g[f"C_{b}"]))
            assert np.array_equal(s.M(b), g[f"M_{b}"])
    assert s.element_status() == (0, 0)


def test_fp64_cube10_matches_oracle():
    mesh, u, p, extra, do_update = cases.cube10_nh()
    s, U, K, F = assemble_state(mesh, u, p, "fp64")
    m, Uo, Ko, Fo = O.solve_state(mesh, u, p, "port")
    assert np.array_equal(U, Uo)
    for b in (1, 12, 2):
        assert rel(K[b], Ko[b]) <= TOL_FP64
    assert rel(F, Fo) <= TOL_FP64


def test_mixed_precision_bounds():
    mesh, u, p, extra, do_update = cases.cube10_nh()
    _, _, K64, F64 = assemble_state(mesh, u, p, "fp64")
    _, _, K32, F32 = assemble_state(mesh, u, p, "mixed")
    assert rel(F32, F64) <= TOL_FP64       # residual stays FP64
    assert rel(K32[2], K64[2]) <= TOL_MIXED_K
    assert rel(K32[2], K64[2]) > 0.0       # the tangent really ran in FP32


SOLID81_CASES = ["cube3_nh", "cube4_nh_clamped", "mr_twist_3x2x4", "biderman_3x3x3_clamped",
                 "bar_mpc_2x2x3", "ce_block_3x3x2", "bar_mpc_ce_2x2x3"]


@pytest.mark.parametrize("name", SOLID81_CASES)
def test_mixed_matches_reference_fixtures(name):
    """The mixed path against the reference's own dumps, per material
    (Neo-Hookean, Mooney-Rivlin, Biderman), with rigid-body and linear MPCs:
    the float-pair residual within the FP64 bound, the FP32 tangent within
    TOL_MIXED_K."""
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    s, U, K, F = _gpu(cases.FULL_CASES[name], "mixed")
    assert np.array_equal(U, g["U"])
    assert rel(F, g["F"]) <= TOL_FP64, rel(F, g["F"])
    for b in (1, 12, 2):
        assert rel(K[b], g[f"K_{b}"]) <= TOL_MIXED_K, (b, rel(K[b], g[f"K_{b}"]))
    assert s.element_status() == (0, 0)


def _entry_classes(s):
    """Per K block: a class per stored entry, 0 = displacement-displacement
    (K_uu), 1 = pressure-displacement (K_up), 2 = pressure-pressure (K_pp),
    3 = a row or column of an MPC equation.  Block-local indices are mapped
    back to equations (block(1): constrained, block(1,2): constrained x the
    rest, block(2): the rest; BlockSparseMatrix.h:126-168)."""
    ne, ee = s.eq_numbers()
    pres = np.zeros(s.n_total + 1, bool)
    pe = ee[:, mg.HYDRO_PRESSURE].astype(np.int64)
    pres[pe[pe > 0]] = True
    mpc = np.zeros(s.n_total + 1, bool)
    mpc[s.n_dofs + 1:] = True
    out = {}
    for b, (ro, co) in {1: (0, 0), 12: (0, s.n_con), 2: (s.n_con, s.n_con)}.items():
        io, cols = s.pattern(b)
        rows = np.repeat(np.arange(1, io.size, dtype=np.int64), np.diff(io.astype(np.int64)))
        r = rows + ro
        c = cols.astype(np.int64) + co
        cls = pres[r].astype(np.int8) + pres[c].astype(np.int8)
        cls[mpc[r] | mpc[c]] = 3
        out[b] = cls
    return out, pres


def _rel_masked(a, b, m):
    return rel(a[m], b[m]) if m.any() else 0.0


@pytest.mark.parametrize("name", SOLID81_CASES)
def test_mixed_volumetric_terms_fp64(name):
    """The mixed path keeps FP64 for the volumetric terms: the pressure
    coupling K_up (D_p = J C^-1), K_pp and the pressure rows F_p of F
    (J - 1 - p/K) within the FP64 bound of the reference's dumps, K_uu within
    TOL_MIXED_K; the MPC rows are FP64 in both precisions."""
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    s, U, K, F = _gpu(cases.FULL_CASES[name], "mixed")
    cls, pres = _entry_classes(s)
    seen = set()
    for b in (1, 12, 2):
        ref = g[f"K_{b}"]
        for c, tol in ((0, TOL_MIXED_K), (1, TOL_FP64), (2, TOL_FP64), (3, TOL_FP64)):
            m = cls[b] == c
            if m.any():
                seen.add(c)
            assert _rel_masked(K[b], ref, m) <= tol, (b, c, _rel_masked(K[b], ref, m))
    assert {0, 1, 2} <= seen
    fp = pres[1:F.size + 1]
    assert fp.any()
    assert _rel_masked(F, g["F"], fp) <= TOL_FP64, _rel_masked(F, g["F"], fp)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_run_to_run_bitwise_reproducible(precision):
    mesh, u, p, extra, do_update = cases.cube4_nh_clamped()
    s = FEStorage(mesh, precision).initSolutionData()
    ne, ee = s.eq_numbers()
    s.setU(mg.u_to_vector(ne, ee, u, p, s.n_total))
    s.updateResults()
    s.assembleGlobalEqMatrices()
    first = [s.K(b).copy() for b in (1, 12, 2)] + [s.F().copy()]
    for _ in range(3):
        s.assembleGlobalEqMatrices()
        again = [s.K(b) for b in (1, 12, 2)] + [s.F()]
        for x, y in zip(first, again):
            assert np.array_equal(x.view(np.uint64), y.view(np.uint64))


@pytest.mark.parametrize("name,precision", [("cube4_nh_clamped", "fp64"),
                                            ("cube4_nh_clamped", "mixed"),
                                            ("bar_mpc_2x2x3", "fp64"),
                                            ("tetra0_3x3x3", "fp64"),
                                            ("quadth_5x4", "fp64"),
                                            ("quadth_lines_6x5", "fp64"),
                                            ("quadth_transient_5x4", "fp64")])
def test_contribution_layouts_bitwise_equal(name, precision):
    """Element-ordered and slot-ordered contributions sum each slot in the
    same order, so K and F agree to the bit."""
    mesh, u, p, extra, do_update = cases.FULL_CASES[name]()
    out = []
    for layout in (0, 1):
        s = FEStorage(mesh, precision).initSolutionData()
        s.set_contrib_layout(layout)
        ne, ee = s.eq_numbers()
        s.setU(mg.u_to_vector(ne, ee, u, p, s.n_total, extra))
        if do_update:
            s.updateResults()
        s.assembleGlobalEqMatrices()
        out.append([s.K(b).copy() for b in (1, 12, 2)] + [s.F().copy()] +
                   ([s.C(b) for b in (1, 12, 2)] if s.transient else []))
    for x, y in zip(*out):
        assert np.array_equal(x.view(np.uint64), y.view(np.uint64))


def test_fresh_state_and_stale_state_semantics():
    """assemble() before any updateResults() uses the Element::pre() state
    (C = I, S = 0); after updateResults(U1), a new U2 changes only the
    pressure read by buildK (SOLID81.cpp:48) -- exactly as the reference."""
    mesh, u, p, _, _ = cases.cube3_nh()
    o = O.OracleModel(mesh, "port")
    s = FEStorage(mesh).initSolutionData()
    ne, ee = s.eq_numbers()
    U1 = mg.u_to_vector(ne, ee, u, p, s.n_total)
    # fresh
    o.set_U(U1); o.assemble()
    s.setU(U1); s.assembleGlobalEqMatrices()
    assert rel(s.K(2), o.K(2)) <= TOL_FP64 and rel(s.F(), o.F()) <= TOL_FP64
    # stale: update with U1, assemble with U2
    U2 = mg.u_to_vector(ne, ee, 0.5 * u, p + 0.05, s.n_total)
    o.update(); o.set_U(U2); o.assemble()
    s.updateResults(); s.setU(U2); s.assembleGlobalEqMatrices()
    assert rel(s.K(2), o.K(2)) <= TOL_FP64 and rel(s.F(), o.F()) <= TOL_FP64


@pytest.mark.parametrize("mat", [(mg.MAT_NEO_HOOKEAN, (1.3, 700.0)),
                                 (mg.MAT_MOONEY_RIVLIN, (0.4, 0.1, 2000.0)),
                                 (mg.MAT_BIDERMAN, (0.4, 0.03, 0.002, 0.05, 900.0))])
def test_fp64_materials_twist_vs_oracle(mat):
    mesh = mg.solid81_block(6, 5, 7, 0.2, mat[0], mat[1], clamp_z0=True)
    u, p = mg.twist_state(mesh, angle_deg=25.0, stretch=1.4, noise_frac=0.01, seed=9)
    _, _, K, F = assemble_state(mesh, u, p, "fp64")
    _, _, Ko, Fo = O.solve_state(mesh, u, p, "port")
    for b in (1, 12, 2):
        assert rel(K[b], Ko[b]) <= TOL_FP64
    assert rel(F, Fo) <= TOL_FP64


def test_element_status_flags_inverted_element():
    mesh, u, p, _, _ = cases.cube3_nh()
    u = u.copy()
    # fold node 14 (an interior node) far through its neighbours: J <= 0 nearby
    u[13] = [-3.0, -3.0, -3.0]
    s, _, K, F = assemble_state(mesh, u, p, "fp64")
    count, first = s.element_status()
    assert count > 0 and 1 <= first <= mesh.n_elems
    # the mixed kernel (float-pair J, float det F) flags the same elements
    sm, _, _, _ = assemble_state(mesh, u, p, "mixed")
    assert sm.element_status() == (count, first)


def test_larger_mesh_properties():
    """40^3 twisted Mooney-Rivlin block: free body => sum of internal nodal
    forces ~ 0; FP64 vs port at 1e-12 on the full K."""
    mesh, u, p = mg.config_twist(n=24, seed=4)
    s, U, K, F = assemble_state(mesh, u, p, "fp64")
    ne, ee = s.eq_numbers()
    for d in range(3):
        fd = F[ne[:, d].astype(np.int64) - 1]
        assert abs(fd.sum()) <= 1e-12 * np.abs(fd).sum() * 10
    _, _, Ko, Fo = O.solve_state(mesh, u, p, "port")
    assert rel(K[2], Ko[2]) <= TOL_FP64 and rel(F, Fo) <= TOL_FP64
    # mixed: the float-pair residual on the same twisted block (the gradient
    # from relative displacements keeps it within the FP64 bound)
    _, _, Km, Fm = assemble_state(mesh, u, p, "mixed")
    assert rel(Fm, Fo) <= TOL_FP64 and rel(Km[2], Ko[2]) <= TOL_MIXED_K


@pytest.mark.parametrize("name,precision", [("cube4_nh_clamped", "fp64"),
                                            ("cube4_nh_clamped", "mixed"),
                                            ("bar_mpc_2x2x3", "fp64"),
                                            ("ce_block_3x3x2", "fp64"),
                                            ("tetra0_3x3x3", "fp64"),
                                            ("quadth_transient_5x4", "fp64"),
                                            ("twist16", "fp64"), ("twist16", "mixed")])
def test_assemble_to_host_equals_assemble_then_copy(name, precision):
    """nla3d_assemble_to_host (element ranges, each finished K prefix copied
    while the next range computes) gives the blocks and F of nla3d_assemble +
    nla3d_get_K / nla3d_get_F bit for bit, for any number of ranges."""
    if name == "twist16":
        # large enough (632k K slots) for runs to be copied after early ranges
        mesh, u, p = mg.config_twist(n=16, seed=3)
        extra, do_update = None, True
    else:
        mesh, u, p, extra, do_update = cases.FULL_CASES[name]()
    s = FEStorage(mesh, precision).initSolutionData()
    ne, ee = s.eq_numbers()
    s.setU(mg.u_to_vector(ne, ee, u, p, s.n_total, extra))
    if do_update:
        s.updateResults()
    s.assembleGlobalEqMatrices()
    want = [s.K(b) for b in (1, 12, 2)] + [s.F()]
    wantC = [s.C(b) for b in (1, 12, 2)] if s.transient else []
    for n_chunks in (1, 3, 8, 64):
        got = [np.full(s.blocks[b][2], np.nan) for b in (1, 12, 2)] + [np.full(s.n_total, np.nan)]
        s.assemble_to_host(*got, n_chunks=n_chunks)
        gotC = [s.C(b) for b in (1, 12, 2)] if s.transient else []
        for x, y in zip(want + wantC, got + gotC):
            assert np.array_equal(x.view(np.uint64), y.view(np.uint64)), n_chunks


@pytest.mark.parametrize("transient", [False, True])
def test_thermal_plate_with_lines_vs_oracle(transient):
    """A 40x30 QUADTH plate with volume flux, convection and flux lines (and
    the capacity matrix when transient) against the oracle at 1e-12.  A
    context with surface lines builds its pattern on the host even when the
    device builder is asked for."""
    mesh = mg.quadth_thermal_plate(40, 30, 0.05, seed=7, transient=transient)
    for builder in ("host", "device"):
        s = FEStorage(mesh).set_pattern_builder(builder).initSolutionData()
        assert not s.pattern_on_device()
        o = O.OracleModel(mesh, "port")
        U = np.random.default_rng(2).standard_normal(s.n_total)
        s.setU(U)
        s.assembleGlobalEqMatrices()
        o.set_U(U)
        o.assemble()
        for b in (1, 12, 2):
            assert np.array_equal(s.pattern(b)[1], o.pattern(b)[1])
            assert rel(s.K(b), o.K(b)) <= TOL_FP64
            if transient:
                assert rel(s.C(b), o.C(b)) <= TOL_FP64
                assert not np.any(s.M(b))
        assert rel(s.F(), o.F()) <= TOL_FP64
